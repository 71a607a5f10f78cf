"""Serving loop (continuous batching): requests of mixed sizes submitted
while others are running must each produce exactly the product computed
alone (tolerance 0) and the GMP product, oversized requests are refused,
stop() drains."""
import time

import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart

pytestmark = pytest.mark.gpu


def test_serving_mix_equals_alone(engine):
    rng = np.random.default_rng(2024)
    srv = engine.Server(slots=3, slot_log=20)
    try:
        reqs = []
        for burst in range(2):
            for _ in range(150):
                na = int(2 ** rng.uniform(3, 18))
                nb = int(2 ** rng.uniform(3, 18))
                a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
                b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
                da, db, dc = cudart.DeviceBuffer(4 * na), cudart.DeviceBuffer(4 * nb), cudart.DeviceBuffer(4 * (na + nb))
                da.upload(a)
                db.upload(b)
                t = srv.submit(dc.ptr, da.ptr, na, db.ptr, nb)
                reqs.append((t, a, b, da, db, dc))
            time.sleep(0.01)   # the second burst arrives while the first is on the GPU
        for t, *_ in reqs:
            srv.wait(t, 120.0)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["device_errors"] == 0
        for t, a, b, da, db, dc in reqs:
            state, lat = srv.query(t)
            assert state == 2 and lat > 0
            got = dc.download(np.uint32, len(a) + len(b))
            assert np.array_equal(got, engine.mul(a, b)), t      # the same product computed alone
            want = oracle.gmp_mul(a, b) if oracle.gmp_available() else oracle.mul(a, b)
            assert np.array_equal(got[:len(want)], want) and not got[len(want):].any(), t
        with pytest.raises(engine.EngineError) as ei:
            big = cudart.DeviceBuffer(8)
            srv.submit(big.ptr, big.ptr, 1 << 20, big.ptr, 1 << 20)
        assert ei.value.code == engine.GBNTT_ERR_SIZE
    finally:
        srv.stop()
    for _, _, _, da, db, dc in reqs:
        for buf in (da, db, dc):
            buf.free()
    assert engine.device_errors() == 0


def test_serving_radix3_requests(engine):
    # requests large enough for transforms of 3 2^k points on their own
    # (k >= 20), power-of-two ones of the same sizes and small ones, in one
    # stream of submissions: every product equals GMP's
    rng = np.random.default_rng(77)
    srv = engine.Server(slots=2, slot_log=24)
    with pytest.raises(engine.EngineError):   # the server's requests are sized for the prime set
        engine.set_prime_set(3)
    assert engine.prime_set() == 2
    sizes = [(3 << 19, 3 << 19), ((3 << 20) - 7, 3 << 20), ((1 << 21) + 1, 1 << 21), (1 << 21, (1 << 21) - 1),
             (3 << 19, 1000), (500, 700), (3 << 18, 3 << 18), (40000, 3 << 20)]
    reqs = []
    try:
        for na, nb in sizes:
            a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
            b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
            da, db, dc = cudart.DeviceBuffer(4 * na), cudart.DeviceBuffer(4 * nb), cudart.DeviceBuffer(4 * (na + nb))
            da.upload(a)
            db.upload(b)
            reqs.append((srv.submit(dc.ptr, da.ptr, na, db.ptr, nb), a, b, da, db, dc))
        for t, *_ in reqs:
            srv.wait(t, 120.0)
        assert srv.stats()["device_errors"] == 0
        for t, a, b, da, db, dc in reqs:
            got = dc.download(np.uint32, len(a) + len(b))
            want = oracle.gmp_mul(a, b) if oracle.gmp_available() else oracle.mul(a, b)
            assert np.array_equal(got[:len(want)], want) and not got[len(want):].any(), (len(a), len(b))
    finally:
        srv.stop()
    for _, _, _, da, db, dc in reqs:
        for buf in (da, db, dc):
            buf.free()
    assert engine.device_errors() == 0
