"""The drop-in at the reference's own call sites, as far as it can be shown
without running them on a GPU: the reference's compute_e application
(ntt/app/compute_e/main.c with the unmodified arith layer, bigint.c,
multiply.c, newton.c, base_convert.c), its GMP oracle test
(test_gmp_oracle.c) and its wrap-guard death test (test_wrap_guard.c) are
compiled by path from the reference checkout and linked against
libgbntt.so in place of the HIP engine or ntt_stub.c
(ntt/app/compute_e/Makefile:252-283), with --no-undefined. Every engine
symbol they import must then come from libgbntt.so, and the library must
define every symbol of the reference stub set (ntt_stub.c:19-31).

Running these binaries needs a GPU machine that also has the reference
sources and a compiler for it; the GPU machines here have no copy of the
reference, so the callers' behaviour (aliasing, squaring, managed and
undersized outputs, the size guard) is tested through the same C ABI by
tests/test_gpu_bigint.py."""
import ctypes
import os
import subprocess

import pytest

from oracle import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB_SET = ("ntt_bigint_mul", "ntt_mul_init_impl", "ntt_mul_teardown_impl", "ntt_get_gpu_dispatch_count",
            "ntt_gpu_emergency_reset")


def _imports(exe):
    out = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_reference_callers_link_against_the_library(built_lib):
    r = build.build_ref_dropin(os.path.join(ROOT, "cryptography_gb300"))
    if r is None:
        pytest.skip("reference checkout not present")
    exes, _ = r
    for name in STUB_SET:
        assert hasattr(built_lib, name), name
    for name, exe in exes.items():
        assert os.path.exists(exe), name
        imported = {s for s in _imports(exe) if s.startswith("ntt_")}
        assert imported, name
        assert imported <= set(STUB_SET), (name, imported - set(STUB_SET))
        for sym in imported:
            assert hasattr(built_lib, sym), (name, sym)
    # compute_e reaches all five engine entry points (main.c:58, :243, :325
    # and multiply.c:87, :97-98)
    assert {s for s in _imports(exes["compute_e_gb300"]) if s.startswith("ntt_")} == set(STUB_SET)


def test_reference_limb112_build_links_against_the_112_library(built_lib):
    # The reference's LIMB_BITS=112 BigInt build (ntt/lib/arith/bigint.h:30-43)
    # of compute_e and test_wrap_guard, compiled by path with -DLIMB_BITS=112,
    # links against libgbntt112.so (the same entry points for 16-byte limbs).
    lib112 = os.path.join(ROOT, "cryptography_gb300", "libgbntt112.so")
    assert os.path.exists(lib112)
    r = build.build_ref_dropin(os.path.join(ROOT, "cryptography_gb300"), limb_bits=112)
    if r is None:
        pytest.skip("reference checkout not present")
    exes, _ = r
    lib = ctypes.CDLL(lib112)
    for name, exe in exes.items():
        imported = {s for s in _imports(exe) if s.startswith("ntt_")}
        assert imported and imported <= set(STUB_SET), (name, imported)
        for sym in imported:
            assert hasattr(lib, sym), (name, sym)
    assert {s for s in _imports(exes["compute_e_limb112_gb300"]) if s.startswith("ntt_")} == set(STUB_SET)
