"""CPU tests of the C-ABI library: it builds for sm_103a, loads without a
GPU, and exports every function include/gbntt.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from cryptography_gb300 import engine

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbntt.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    skip = {"sizeof", "defined", "if"}
    return sorted({n for n in names if n not in skip and not n.isupper()})


def test_header_declares_expected_api():
    names = declared_functions()
    for n in ("ntt_mul_init_impl", "ntt_mul_teardown_impl", "ntt_bigint_mul", "ntt_get_gpu_dispatch_count",
              "ntt_gpu_emergency_reset", "bigint_alloc_managed", "hip_free_limbs", "gbntt_mul_u32"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in declared_functions() if not hasattr(built_lib, n)]
    assert not missing, missing
    assert set(declared_functions()) == set(engine.EXPORTS)


def test_limb112_library_exports_the_same_symbols(built_lib):
    # libgbntt112.so: the reference entry points for 112-bit limbs
    # (include/gbntt_limb112.h) plus the same native API
    lib = ctypes.CDLL(os.path.join(os.path.dirname(HEADER), "..", "cryptography_gb300", "libgbntt112.so"))
    h112 = open(os.path.join(os.path.dirname(HEADER), "gbntt_limb112.h")).read()
    h112 = re.sub(r"/\*.*?\*/", "", h112, flags=re.S)
    names = set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", h112)) - {"sizeof"}
    assert {"ntt_mul_init_impl", "ntt_bigint_mul", "bigint_alloc_managed", "ntt_bigint_mul_checked"} <= names
    missing = [n for n in sorted(names | set(declared_functions())) if not hasattr(lib, n)]
    assert not missing, missing


def test_library_is_native_sm103a(built_lib):
    # the library links the CUDA runtime; nothing of the oracle is linked in
    path = engine.lib_path()
    blob = open(path, "rb").read()
    assert b"oracle_" not in blob
    assert b"sm_103a" in blob or b"sm_103" in blob


def test_pure_host_queries(built_lib):
    # no device needed: planning and sizing are host logic
    assert engine.plan(29) == [7, 7, 7, 8]
    assert engine.plan(30) == [7, 7, 8, 8]
    assert engine.plan(21) == [6, 7, 8]
    assert engine.plan(14) == [6, 8]
    assert engine.plan(12) == [6, 6]
    assert engine.plan(5) == [5]
    assert engine.transform_log(1 << 28, 1 << 28) == 29
    assert engine.transform_log(1, 1) == 5
    assert engine.transform_log(1 << 20, 1 << 20) == 21
    assert engine.workspace_bytes(29) > 6 * 8 * (1 << 29)
    assert not engine.is_ready()
    rc = built_lib.gbntt_mul_u32(ctypes.c_void_p(8), ctypes.c_void_p(8), 1, ctypes.c_void_p(8), 1, None)
    assert rc == engine.GBNTT_ERR_NOT_INIT


def test_plan_overrides_host_logic(built_lib):
    # plan overrides are host state: up to four passes of 2^5 .. 2^10 points
    # summing to the transform log; anything else is rejected
    default = engine.plan(29)
    try:
        engine.set_plan(29, [8, 7, 7, 7])
        assert engine.plan(29) == [8, 7, 7, 7]
        for bad in ([5, 6, 6, 6, 6], [10, 10, 8], [4, 10, 10, 5], [11, 9, 9]):
            with pytest.raises(engine.EngineError):
                engine.set_plan(29, bad)
        assert engine.plan(29) == [8, 7, 7, 7]
    finally:
        engine.set_plan(29, [])
    assert engine.plan(29) == default


def test_default_plans_are_valid_factorisations(built_lib):
    # every transform length the engine accepts has a default plan of 1-4
    # passes of 2^5..2^10 points summing to it, smallest lengths in one pass
    for log_n in range(5, 31):
        p = engine.plan(log_n)
        assert 1 <= len(p) <= 4 and sum(p) == log_n, (log_n, p)
        assert all(5 <= x <= 10 for x in p), (log_n, p)
        if log_n <= 10:
            assert p == [log_n]
