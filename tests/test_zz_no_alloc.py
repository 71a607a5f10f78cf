"""gbntt_mul_u32_noalloc: the multiply entry point that allocates nothing.

It exists for callers that cannot allocate device memory where they need a
product (for example an application whose device allocator is owned by a
pool that forbids cudaMalloc/cudaFree, or a latency-critical loop where an
allocation would synchronise the device). Its scratch is one static device
array set up on the first call. This file is collected last so a run that
stops at the first failure has already run every other test; it also passes
alone in a fresh process (the engine fixture initialises the engine it
compares against)."""
import numpy as np
import pytest

from cryptography_gb300 import cudart

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_engine_two_calls(engine):
    lib = engine.lib()
    rng = np.random.default_rng(77)
    cases = [(5000, 3001), (40000, 25000), (1, 1), (65536, 1)]
    for na, nb in cases:
        a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        first = _noalloc(lib, a, b)
        second = _noalloc(lib, a, b)            # the shared scratch keeps the last call's contents
        want = engine.mul(a, b)                 # the existing entry point
        assert np.array_equal(first, want), (na, nb)
        assert np.array_equal(second, want), (na, nb)
    sq = rng.integers(0, 1 << 32, 30000, dtype=np.uint64).astype(np.uint32)
    assert np.array_equal(_noalloc(lib, sq, sq), engine.mul(sq, sq))


def test_noalloc_rejects_oversize(engine):
    lib = engine.lib()
    da, dc = cudart.DeviceBuffer(8), cudart.DeviceBuffer(8)
    # (2^16 + 1) coefficients needed: above the stated maximum, rejected on the host
    rc = lib.gbntt_mul_u32_noalloc(dc.ptr, da.ptr, 40000, da.ptr, 25538, None)
    assert rc == engine.GBNTT_ERR_SIZE
    da.free()
    dc.free()
