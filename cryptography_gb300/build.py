"""Build recipe for the CUDA libraries ``libgbntt.so`` and ``libgbntt112.so``
(sm_103a only).

Compiles each translation unit with nvcc in parallel and links the shared
libraries in-tree next to this file: ``libgbntt.so`` carries the reference
entry points for 64-bit BigInt limbs, ``libgbntt112.so`` the same symbols for
the reference's 112-bit limb build (``gbntt_refabi.cu`` compiled a second time
with ``GBNTT_LIMB_BITS=112``); every other object is shared. Invoked by
``__graft_entry__.build()`` and on first import when a library is missing or
older than its sources.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbntt.so")
LIB112 = os.path.join(HERE, "libgbntt112.so")

SOURCES = ["gbntt_pass_p0.cu", "gbntt_pass_p1.cu", "gbntt_pass_p2.cu", "gbntt_pass_p3.cu", "gbntt_pass_p4.cu", "gbntt_kernels.cu", "gbntt_engine.cu", "gbntt_noalloc.cu",
           "gbntt_e.cu", "gbntt_negacyclic.cu", "gbntt_refabi.cu", "gbntt_radix3.cu"]
# (source, object name, extra flags): the reference entry points once more for 112-bit limbs
VARIANTS = [("gbntt_refabi.cu", "gbntt_refabi112", ["-DGBNTT_LIMB_BITS=112"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")


def _cuda_lib_dir():
    home = os.environ.get("CUDA_HOME") or os.path.dirname(os.path.dirname(os.path.realpath(
        subprocess.run(["which", NVCC], capture_output=True, text=True).stdout.strip() or "/usr/local/cuda/bin/nvcc")))
    return os.path.join(home, "lib64")


def _flags():
    extra = []
    if os.environ.get("GBNTT_PASS_MIN_BLOCKS"):   # tuning knob: resident CTAs per SM of the pass kernels
        extra.append("-DGBNTT_PASS_MIN_BLOCKS=%d" % int(os.environ["GBNTT_PASS_MIN_BLOCKS"]))
    if os.environ.get("GBNTT_PASS_SHARED_DFT"):
        extra.append("-DGBNTT_PASS_SHARED_DFT=%d" % int(os.environ["GBNTT_PASS_SHARED_DFT"]))
    for knob in ("GBNTT_PASS_PIPE32", "GBNTT_PASS_PIPE64", "GBNTT_PASS_PW_ASYNC", "GBNTT_Q0_ALU", "GBNTT_P3_ALU", "GBNTT_CARRY_MIN_BLOCKS", "GBNTT_PASS_MIN_BLOCKS_SMALL", "GBNTT_Q0_POW2", "GBNTT_FUSED_MIN_BLOCKS",
                 "GBNTT_PASS_LIMB_ASYNC"):
        if os.environ.get(knob):
            extra.append("-D%s=%d" % (knob, int(os.environ[knob])))
    if os.environ.get("GBNTT_PASS_CPASYNC"):
        extra.append("-DGBNTT_PASS_CPASYNC=%d" % int(os.environ["GBNTT_PASS_CPASYNC"]))
    if os.environ.get("GBNTT_PASS_MIN_BLOCKS32"):
        extra.append("-DGBNTT_PASS_MIN_BLOCKS32=%d" % int(os.environ["GBNTT_PASS_MIN_BLOCKS32"]))
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                   "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr"] + extra


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + \
        [os.path.join(INCLUDE, f) for f in ("gbntt.h", "gbntt_limb112.h")] + [__file__]


def stale():
    if not os.path.exists(LIB) or not os.path.exists(LIB112) or os.environ.get("GBNTT_FORCE_BUILD"):
        return True
    t = min(os.path.getmtime(LIB), os.path.getmtime(LIB112))
    return any(os.path.getmtime(d) > t for d in _deps())


def _compile(src, verbose, name=None, extra=()):
    obj = os.path.join(BUILD_DIR, (name or os.path.splitext(src)[0]) + ".o")
    cmd = [NVCC] + _flags() + list(extra) + (["-Xptxas", "-v"] if verbose else []) + \
        ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False):
    if not force and not stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    jobs = [(s, None, ()) for s in SOURCES] + list(VARIANTS)
    with concurrent.futures.ThreadPoolExecutor(len(jobs)) as ex:
        results = list(ex.map(lambda j: _compile(j[0], verbose, j[1], j[2]), jobs))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    shared = objs[:len(SOURCES)]
    ref64 = os.path.join(BUILD_DIR, "gbntt_refabi.o")
    ref112 = objs[len(SOURCES)]
    for lib, ref in ((LIB, ref64), (LIB112, ref112)):
        tmp = lib + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "--cudart", "shared", "-Xlinker", "-rpath=" + _cuda_lib_dir(), "-o", tmp] + \
            [o for o in shared if o != ref64] + [ref]
        subprocess.check_call(cmd)
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose="-v" in sys.argv))
