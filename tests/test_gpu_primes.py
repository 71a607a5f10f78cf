"""The two prime sets for 32-bit coefficients: q0 + the 32-bit p3 (default)
and the reference's three 64-bit primes. Every product must be identical
under both, and equal to GMP, including the largest coefficients (all-ones
operands) at transform lengths up to the engine's maximum and the batched
path; the set switch is host logic with argument checks."""
import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart, synth

pytestmark = pytest.mark.gpu


def _gmp(a, b):
    c = oracle.gmp_mul(a, b)
    out = np.zeros(len(a) + len(b), dtype=np.uint32)
    out[:len(c)] = c
    return out


def _both(engine, a, b):
    engine.set_prime_set(3)
    try:
        c3 = engine.mul(a, b)
    finally:
        engine.set_prime_set(2)
    c2 = engine.mul(a, b)
    return c2, c3


def test_default_is_two_primes(engine):
    assert engine.prime_set() == 2
    with pytest.raises(engine.EngineError):
        engine.set_prime_set(4)
    assert engine.prime_set() == 2


@pytest.mark.parametrize("log_n", [5, 6, 10, 11, 15, 20, 21, 24])
def test_sets_agree_at_length_boundaries(engine, log_n):
    rng = np.random.default_rng(300 + log_n)
    N = 1 << log_n
    for need in (N, N - 1):
        na = need // 2 + 1
        nb = need + 1 - na
        a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        c2, c3 = _both(engine, a, b)
        assert np.array_equal(c2, c3), (log_n, need)
        if log_n <= 21:
            assert np.array_equal(c2, _gmp(a, b)), (log_n, need)
    assert engine.device_errors() == 0


def test_largest_coefficients(engine):
    # all-ones operands give coefficients near min(na, nb) * (2^32 - 1)^2,
    # the CRT bound's worst case; the longest product of the engine
    for n in (1, 2, 1000, 1 << 16, (1 << 23) - 1):
        a = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
        v = (1 << (32 * n)) - 1
        got = engine.mul(a, a)
        if n <= (1 << 16):
            assert oracle.to_int(got) == v * v, n
        else:
            # (2^k - 1)^2 = 2^2k - 2^(k+1) + 1: limb 0 = 1, limbs 1..n-1 = 0,
            # limb n = 0xFFFFFFFE, limbs n+1..2n-1 = all ones
            assert got[0] == 1 and not got[1:n].any() and got[n] == 0xFFFFFFFE
            assert (got[n + 1:] == 0xFFFFFFFF).all()
    assert engine.device_errors() == 0


def test_squares_and_random_sizes(engine):
    rng = np.random.default_rng(31)
    for na, nb in [(1, 1), (3, 1), (17, 33), (1000, 999), (4097, 3), (70000, 12345), (1 << 20, 1 << 20)]:
        a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        c2, c3 = _both(engine, a, b)
        assert np.array_equal(c2, c3), (na, nb)
        s2, s3 = _both(engine, a, a)
        assert np.array_equal(s2, s3), na
    assert engine.device_errors() == 0


def test_batched_two_prime_matches_single(engine):
    rng = np.random.default_rng(32)
    A = [rng.integers(0, 1 << 32, int(n), dtype=np.uint64).astype(np.uint32)
         for n in rng.integers(1, 5000, 200)]
    B = [rng.integers(0, 1 << 32, int(n), dtype=np.uint64).astype(np.uint32)
         for n in rng.integers(1, 5000, 200)]
    da = [cudart.DeviceBuffer(4 * len(a)) for a in A]
    db = [cudart.DeviceBuffer(4 * len(b)) for b in B]
    dc = [cudart.DeviceBuffer(4 * (len(a) + len(b))) for a, b in zip(A, B)]
    for d, a in zip(da, A):
        d.upload(a)
    for d, b in zip(db, B):
        d.upload(b)
    engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                            [x.ptr for x in db], [len(b) for b in B])
    cudart.synchronize()
    for c, a, b in zip(dc, A, B):
        assert np.array_equal(c.download(np.uint32, len(a) + len(b)), engine.mul(a, b))
    for buf in da + db + dc:
        buf.free()
    assert engine.device_errors() == 0


def test_synth_2pow22_both_sets(engine):
    a = synth.operand(1 << 22, 41)
    b = synth.operand(1 << 22, 42)
    c2, c3 = _both(engine, a, b)
    assert np.array_equal(c2, c3)
    assert np.array_equal(c2, _gmp(a, b))


@pytest.mark.parametrize("knobs", [{"GBNTT_Q0_FORM": "lazy"}, {"GBNTT_OVERLAP": "0"},
                                   {"GBNTT_Q0_FORM": "lazy", "GBNTT_OVERLAP": "0"}, {"GBNTT_RADIX3": "0"},
                                   {"GBNTT_Q0_FORM": "lazy", "GBNTT_RADIX3_MIN_LOG": "10"}])
def test_engine_knobs_give_identical_products(knobs):
    # the tuning switches (lazy normal-form q0, no second-prime stream, no
    # transforms of length 3 2^k) change how the product is computed, never
    # its value
    import json
    import os
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    body = textwrap.dedent("""
        import json, sys
        sys.path.insert(0, %r)
        import numpy as np
        import cryptography_gb300 as g
        import oracle
        g.init(22)
        rng = np.random.default_rng(71)
        ok = []
        for na, nb in [(1, 1), (33, 17), (4096, 4095), (70000, 12345), ((1 << 20) + 1, (1 << 20) - 3)]:
            a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
            b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
            want = np.zeros(na + nb, dtype=np.uint32)
            r = oracle.gmp_mul(a, b)
            want[:len(r)] = r
            ok.append(bool(np.array_equal(g.mul(a, b), want)))
        full = np.full((1 << 20) - 1, 0xFFFFFFFF, dtype=np.uint32)
        c = g.mul(full, full)
        n = len(full)
        ok.append(bool(c[0] == 1 and not c[1:n].any() and c[n] == 0xFFFFFFFE and (c[n + 1:] == 0xFFFFFFFF).all()))
        print(json.dumps([ok, g.device_errors()]))
    """ % root)
    env = dict(os.environ, **knobs)
    r = subprocess.run([sys.executable, "-c", body], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    ok, errs = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(ok) and errs == 0, (knobs, ok)
