"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles ``crt_ntt_oracle.c`` (the CPU restatement of the
  reference CRT-NTT multiply) into ``oracle/liboracle.so``.
* ``build_ref()`` compiles the reference's own host sources, by path from the
  reference checkout, together with ``ref_shim.cpp`` into
  ``oracle/_ref/libref.so``. Nothing from the reference is copied; when the
  checkout is absent (machines without it) it is skipped and the tests that need it
  skip too.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libref.so")
# The reference checkout: GBNTT_REFERENCE_ROOT, else a directory named
# "reference" beside this repository's root (absent on machines without it).
REFERENCE_ROOT = os.environ.get("GBNTT_REFERENCE_ROOT") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "crt_ntt_oracle.c")
    if force or _stale(ORACLE_SO, [src, __file__]):
        tmp = ORACLE_SO + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=gnu11",
                               "-Wall", src, "-o", tmp, "-ldl"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


E_ORACLE_SO = os.path.join(HERE, "libeoracle.so")


def build_e_oracle(force=False):
    """Compile e_gmp_oracle.c (the reference's compute_e path on GMP) into
    oracle/libeoracle.so, linked against the system libgmp.so.10."""
    src = os.path.join(HERE, "e_gmp_oracle.c")
    if force or _stale(E_ORACLE_SO, [src, __file__]):
        tmp = E_ORACLE_SO + ".tmp"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11", "-Wall", src, "-o", tmp,
                               "-l:libgmp.so.10", "-lm"])
        os.replace(tmp, E_ORACLE_SO)
    return E_ORACLE_SO


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE_ROOT, "ntt", "lib", "garner.hip"))


def build_ref(force=False):
    """Compile the reference host code (bigint.c, garner.hip host part,
    primes.h, shoup.h) by path. Returns the .so path or None if the
    reference checkout is not present."""
    if not reference_available():
        return None
    lib = os.path.join(REFERENCE_ROOT, "ntt", "lib")
    arith = os.path.join(lib, "arith")
    shim = os.path.join(HERE, "ref_shim.cpp")
    bigint_c = os.path.join(arith, "bigint.c")
    if not (force or _stale(REF_SO, [shim, bigint_c, os.path.join(lib, "garner.hip"), __file__])):
        return REF_SO
    os.makedirs(REF_DIR, exist_ok=True)
    obj = os.path.join(REF_DIR, "bigint.o")
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-c", "-I", lib, "-I", arith,
                           bigint_c, "-o", obj])
    tmp = REF_SO + ".tmp"
    subprocess.check_call(["g++", "-O2", "-fopenmp", "-fPIC", "-shared",
                           "-I", lib, "-I", arith, shim, obj, "-o", tmp])
    os.replace(tmp, REF_SO)
    return REF_SO


REF_E = os.path.join(REF_DIR, "compute_e_ref")


def build_ref_compute_e(force=False):
    """The reference's host compute_e (main.c with -DCOMPUTE_E_HOST, the
    arith layer, binary splitting) linked with ref_e_gmp_shim.c, compiled by
    path from the reference checkout. None when the checkout is absent or
    libgmp.so.10 cannot be linked."""
    if not reference_available():
        return None
    ce = os.path.join(REFERENCE_ROOT, "ntt", "app", "compute_e")
    lib = os.path.join(REFERENCE_ROOT, "ntt", "lib")
    arith = os.path.join(lib, "arith")
    srcs = [os.path.join(ce, f) for f in ("main.c", "binary_split.c", "mem_pool.c")] + \
           [os.path.join(arith, f) for f in ("bigint.c", "multiply.c", "newton.c", "base_convert.c")] + \
           [os.path.join(HERE, "ref_e_gmp_shim.c")]
    if not (force or _stale(REF_E, srcs + [__file__])):
        return REF_E
    os.makedirs(REF_DIR, exist_ok=True)
    objs = []
    for src in srcs:
        obj = os.path.join(REF_DIR, "e_" + os.path.basename(src)[:-2] + ".o")
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-DCOMPUTE_E_HOST=1", "-I", lib, "-I", arith, "-I", ce,
                               "-c", src, "-o", obj])
        objs.append(obj)
    tmp = REF_E + ".tmp"
    subprocess.check_call(["gcc"] + objs + ["-lm", "-fopenmp", "-l:libgmp.so.10", "-o", tmp])
    os.replace(tmp, REF_E)
    return REF_E


# The reference's own callers of the engine, linked against libgbntt.so
# instead of the HIP engine (or ntt_stub.c): compute_e, test_gmp_oracle and
# test_wrap_guard (ntt/app/compute_e/Makefile builds the same objects).
DROPIN_BINARIES = {
    "compute_e_gb300": (["app/compute_e/main.c", "app/compute_e/binary_split.c", "app/compute_e/mem_pool.c",
                         "lib/arith/bigint.c", "lib/arith/multiply.c", "lib/arith/newton.c",
                         "lib/arith/base_convert.c"], ["-lm", "-fopenmp"]),
    "test_gmp_oracle_gb300": (["app/compute_e/test_gmp_oracle.c", "lib/arith/bigint.c", "lib/arith/multiply.c"],
                              ["-l:libgmp.so.10"]),
    "test_wrap_guard_gb300": (["app/compute_e/test_wrap_guard.c", "lib/arith/bigint.c"], []),
}


# the reference's LIMB_BITS=112 build of the same callers (its GMP oracle
# imports 64-bit limbs and is left out), linked against libgbntt112.so
DROPIN_BINARIES_112 = {k.replace("_gb300", "_limb112_gb300"): v for k, v in DROPIN_BINARIES.items()
                       if not k.startswith("test_gmp_oracle")}


def build_ref_dropin(gbntt_dir, force=False, limb_bits=64):
    """Compile the reference's callers by path (the GPU build: no
    COMPUTE_E_HOST, no stub) and link them against gbntt_dir/libgbntt.so,
    or with limb_bits=112 compile them with -DLIMB_BITS=112 and link them
    against gbntt_dir/libgbntt112.so. Returns {binary: path} and the object
    files per binary, or None when the reference checkout is absent. The
    binaries run on a machine with a GPU, the reference sources and a
    compiler for that machine."""
    if not reference_available():
        return None
    ntt = os.path.join(REFERENCE_ROOT, "ntt")
    inc = ["-I", os.path.join(ntt, "lib"), "-I", os.path.join(ntt, "lib", "arith"),
           "-I", os.path.join(ntt, "app", "compute_e")]
    lib = "libgbntt112.so" if limb_bits == 112 else "libgbntt.so"
    so = os.path.join(gbntt_dir, lib)
    defs = ["-DLIMB_BITS=112"] if limb_bits == 112 else []
    tag = "dropin112_" if limb_bits == 112 else "dropin_"
    out, objs_of = {}, {}
    os.makedirs(REF_DIR, exist_ok=True)
    for name, (srcs, libs) in (DROPIN_BINARIES_112 if limb_bits == 112 else DROPIN_BINARIES).items():
        exe = os.path.join(REF_DIR, name)
        paths = [os.path.join(ntt, s_) for s_ in srcs]
        objs = [os.path.join(REF_DIR, tag + os.path.basename(s_)[:-2] + ".o") for s_ in srcs]
        if force or _stale(exe, paths + [so, __file__]):
            for src, obj in zip(paths, objs):
                subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fopenmp"] + defs + inc + ["-c", src, "-o", obj])
            tmp = exe + ".tmp"
            subprocess.check_call(["gcc"] + objs + ["-L", gbntt_dir, "-l:" + lib,
                                                    "-Wl,-rpath," + gbntt_dir, "-Wl,--no-undefined"] + libs +
                                  ["-o", tmp])
            os.replace(tmp, exe)
        out[name] = exe
        objs_of[name] = objs
    return out, objs_of


REF_NEGA_SO = os.path.join(REF_DIR, "libref_nega.so")


def build_ref_negacyclic(force=False):
    """The reference's CPU negacyclic multiply (ntt/ref/ntt_polymul_negacyclic.c,
    library form -DNTT_NEGACYC_NO_MAIN) compiled by path with
    ref_negacyclic_shim.c into oracle/_ref/libref_nega.so. None when the
    reference checkout is absent."""
    if not reference_available():
        return None
    ref = os.path.join(REFERENCE_ROOT, "ntt", "ref")
    src = os.path.join(ref, "ntt_polymul_negacyclic.c")
    shim = os.path.join(HERE, "ref_negacyclic_shim.c")
    if not (force or _stale(REF_NEGA_SO, [src, shim, __file__])):
        return REF_NEGA_SO
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_NEGA_SO + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-DNTT_NEGACYC_NO_MAIN", "-I", ref,
                           src, shim, "-o", tmp])
    os.replace(tmp, REF_NEGA_SO)
    return REF_NEGA_SO


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_e_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_compute_e(force=True))
