"""Negacyclic products mod X^N + 1 (gbntt_negacyclic_mul_u64) against the
oracle's definition at sizes it evaluates in seconds, extreme coefficients
(the largest magnitudes of both signs), squaring, and at sizes beyond the
oracle through exact identities: f * 1 = f and f * X = the shift of f with
its top coefficient negated."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_negacyclic_matches_oracle(engine):
    rng = np.random.default_rng(77)
    for log_n in (5, 6, 9, 12, 15):
        n = 1 << log_n
        f = rng.integers(0, 1 << 64, n, dtype=np.uint64)
        g = rng.integers(0, 1 << 64, n, dtype=np.uint64)
        assert engine.negacyclic_mul(f, g) == oracle.negacyclic_mul(f, g), log_n
    assert engine.device_errors() == 0


def test_negacyclic_matches_reference_cpu_multiply(engine):
    # the reference's own CPU negacyclic multiply (polymul_ntt_negacyclic,
    # ntt/ref/ntt_polymul_negacyclic.c:178-213), recorded on seeded inputs in
    # tests/golden/negacyclic_ref.json: the exact GPU coefficients reduced
    # mod each case's q equal its outputs
    import hashlib
    import json
    import os
    from cryptography_gb300 import synth
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "negacyclic_ref.json")
    cases = json.load(open(path))["cases"]
    for label, c in cases.items():
        n, q = c["n"], c["q"]
        f = (synth.splitmix64(c["seed_f"], 0, n) % np.uint64(q)).astype(np.uint64)
        g = (synth.splitmix64(c["seed_g"], 0, n) % np.uint64(q)).astype(np.uint64)
        got = np.array([v % q for v in engine.negacyclic_mul(f, g)], dtype=np.uint64)
        assert [int(v) for v in got[:8]] == c["head"], label
        assert [int(v) for v in got[-8:]] == c["tail"], label
        assert hashlib.sha256(got.astype("<u8").tobytes()).hexdigest() == c["sha256"], label
    assert engine.device_errors() == 0


def test_negacyclic_extreme_coefficients_and_squares(engine):
    n = 1 << 10
    top = np.full(n, (1 << 64) - 1, dtype=np.uint64)
    assert engine.negacyclic_mul(top, top) == oracle.negacyclic_mul(top, top)
    # one nonzero top coefficient each: a single negative wrap-around term
    e = np.zeros(n, dtype=np.uint64)
    e[n - 1] = (1 << 64) - 1
    got = engine.negacyclic_mul(e, e)
    assert got[n - 2] == -(((1 << 64) - 1) ** 2) and sum(v != 0 for v in got) == 1
    rng = np.random.default_rng(3)
    f = rng.integers(0, 1 << 64, 1 << 11, dtype=np.uint64)
    assert engine.negacyclic_mul(f, f) == oracle.negacyclic_mul(f, f)
    assert engine.device_errors() == 0


@pytest.mark.parametrize("log_n", [20, 24])
def test_negacyclic_identities_at_large_sizes(engine, log_n):
    rng = np.random.default_rng(log_n)
    n = 1 << log_n
    f = rng.integers(0, 1 << 64, n, dtype=np.uint64)
    one = np.zeros(n, dtype=np.uint64)
    one[0] = 1
    got = engine.negacyclic_mul(f, one)
    assert got == [int(v) for v in f]
    x = np.zeros(n, dtype=np.uint64)
    x[1] = 1
    got = engine.negacyclic_mul(f, x)
    assert got[0] == -int(f[-1]) and got[1:] == [int(v) for v in f[:-1]]
    assert engine.device_errors() == 0


def test_negacyclic_rejects_bad_sizes(engine):
    from cryptography_gb300 import cudart
    buf = cudart.DeviceBuffer(32 * 64)
    try:
        for log_n in (4, 30, 25):   # below 2^5, above 2^29, above the engine's 2^24
            with pytest.raises(engine.EngineError):
                engine.negacyclic_mul_device(buf.ptr, buf.ptr, buf.ptr, log_n)
    finally:
        buf.free()
