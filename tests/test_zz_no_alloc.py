"""gbntt_mul_u32_noalloc: the multiply entry point that allocates nothing.

It exists for callers that cannot allocate device memory where they need a
product (for example an application whose device allocator is owned by a
pool that forbids cudaMalloc/cudaFree, or a latency-critical loop where an
allocation would synchronise the device). Its scratch is one static device
array set up on the first call. Products are checked against the CPU
oracle and, on two calls in a row, against the engine's own entry point.
This file is collected last so a run that stops at the first failure has
already run every other test; it also passes alone in a fresh process, and
one test runs the entry point in a child process before any engine exists.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ERR_LOOKBACK_TIMEOUT = 2


def _noalloc(lib, a, b):
    na, nb = len(a), len(b)
    da, db = cudart.DeviceBuffer(4 * na), cudart.DeviceBuffer(4 * nb)
    dc = cudart.DeviceBuffer(4 * (na + nb))
    da.upload(a)
    db.upload(b)
    same = a is b
    rc = lib.gbntt_mul_u32_noalloc(dc.ptr, da.ptr, na, da.ptr if same else db.ptr, nb, None)
    assert rc == 0, rc
    cudart.synchronize()
    out = dc.download(np.uint32, na + nb)
    for buf in (da, db, dc):
        buf.free()
    return out


def _want(a, b):
    want = np.zeros(len(a) + len(b), dtype=np.uint32)
    r = oracle.mul(a, b)
    want[:len(r)] = r
    return want


def test_noalloc_matches_oracle_and_engine_two_calls(engine):
    lib = engine.lib()
    rng = np.random.default_rng(77)
    cases = [(5000, 3001), (40000, 25000), (1, 1), (65536, 1), (1025, 2047)]
    for na, nb in cases:
        a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        first = _noalloc(lib, a, b)
        second = _noalloc(lib, a, b)            # the shared scratch keeps the last call's contents
        want = _want(a, b)
        assert np.array_equal(first, want), (na, nb)
        assert np.array_equal(second, want), (na, nb)
        assert np.array_equal(second, engine.mul(a, b)), (na, nb)   # the existing entry point
    sq = rng.integers(0, 1 << 32, 30000, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(_noalloc(lib, sq, sq), _want(sq, sq))
    ones = np.full(32768, 0xFFFFFFFF, dtype=np.uint32)      # every coefficient at its largest
    assert np.array_equal(_noalloc(lib, ones, ones), _want(ones, ones))
    assert engine.device_errors() == 0


def test_noalloc_rejects_oversize(engine):
    lib = engine.lib()
    da, dc = cudart.DeviceBuffer(8), cudart.DeviceBuffer(8)
    # (2^16 + 1) coefficients needed: above the stated maximum, rejected on the host
    rc = lib.gbntt_mul_u32_noalloc(dc.ptr, da.ptr, 40000, da.ptr, 25538, None)
    assert rc == engine.GBNTT_ERR_SIZE
    da.free()
    dc.free()


def test_noalloc_wait_runs_out_and_reports(engine):
    # a look-back wait in the scratch's carry scan that nothing answers ends
    # by itself; its error bit reaches the host through gbntt_device_errors
    # and stays set until read; the next product is exact
    lib = engine.lib()
    sec = ctypes.c_double(0)
    assert lib.gbntt_debug_noalloc_lookback_timeout(ctypes.byref(sec)) == 0
    assert 0 < sec.value < 30
    assert engine.device_errors() & ERR_LOOKBACK_TIMEOUT
    assert engine.device_errors() == 0
    rng = np.random.default_rng(6)
    a = rng.integers(0, 1 << 32, 9000, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 1 << 32, 7000, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(_noalloc(lib, a, b), _want(a, b))
    assert engine.device_errors() == 0


_CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import oracle
from cryptography_gb300 import cudart, engine
lib = engine.lib()
assert not engine.is_ready()
rng = np.random.default_rng(11)
for na, nb in ((20000, 13000), (3, 65534)):
    a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
    da, db, dc = cudart.DeviceBuffer(4 * na), cudart.DeviceBuffer(4 * nb), cudart.DeviceBuffer(4 * (na + nb))
    da.upload(a)
    db.upload(b)
    for rep in range(2):
        assert lib.gbntt_mul_u32_noalloc(dc.ptr, da.ptr, na, db.ptr, nb, None) == 0
        cudart.synchronize()
        got = dc.download(np.uint32, na + nb)
        want = np.zeros(na + nb, dtype=np.uint32)
        r = oracle.mul(a, b)
        want[:len(r)] = r
        assert np.array_equal(got, want), (na, nb, rep)
assert engine.device_errors() == 0
assert not engine.is_ready()
print("CHILD_OK")
"""


def test_noalloc_without_engine_in_fresh_process(built_lib):
    # the entry point needs no gbntt_init: a fresh process that never
    # initialises the engine multiplies through it alone
    r = subprocess.run([sys.executable, "-c", _CHILD, ROOT], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "CHILD_OK" in r.stdout
