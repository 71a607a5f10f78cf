"""The plan autotuner: every installed plan is a valid factorisation, the
timings are positive, and products stay exact under the tuned plans (then the
default plans are restored for the other tests)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def test_autotune_installs_valid_plans_and_keeps_products_exact(engine):
    lo, hi = 5, 17
    try:
        res = engine.autotune(lo, hi, reps=2)
        assert sorted(res) == list(range(lo, hi + 1))
        for L, (plan, ms) in res.items():
            assert 1 <= len(plan) <= 4 and sum(plan) == L, (L, plan)
            assert all(5 <= p <= 10 for p in plan), (L, plan)
            assert ms > 0
            assert engine.plan(L) == plan
        rng = np.random.default_rng(17)
        for na, nb in [(1, 1), (17, 16), (300, 211), (2048, 2049), (40000, 25000), (65536, 65535)]:
            a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
            b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
            want = np.zeros(na + nb, dtype=np.uint32)
            r = oracle.mul(a, b)
            want[:len(r)] = r
            assert np.array_equal(engine.mul(a, b), want), (na, nb)
        assert engine.device_errors() == 0
    finally:
        for L in range(lo, hi + 1):
            engine.set_plan(L, [])


def test_autotune_rejects_bad_ranges(engine):
    with pytest.raises(engine.EngineError):
        engine.autotune(4, 10)
    with pytest.raises(engine.EngineError):
        engine.autotune(12, 11)
    with pytest.raises(engine.EngineError):
        engine.autotune(5, engine.lib().gbntt_max_log() + 1)


@pytest.mark.parametrize("log_n,plan", [(20, [5, 5, 5, 5]), (22, [6, 5, 6, 5]), (24, [6, 6, 6, 6]),
                                        (23, [5, 8, 5, 5]), (21, [10, 6, 5]), (18, [9, 9])])
def test_hand_set_plans_give_exact_products(engine, log_n, plan):
    # four-pass plans (and other factorisations) set by hand: products of
    # every shape must stay exact (GMP), in both operand orders, and squares
    rng = np.random.default_rng(log_n * 7 + len(plan))
    N = 1 << log_n
    try:
        engine.set_plan(log_n, plan)
        assert engine.plan(log_n) == plan
        for na, nb in [(N // 2 + 1, N // 2 - 1), (N - 40, 40), (N // 4 + 5, N // 2)]:
            a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
            b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
            want = np.zeros(na + nb, dtype=np.uint32)
            r = oracle.gmp_mul(a, b)
            want[:len(r)] = r
            assert np.array_equal(engine.mul(a, b), want), (na, nb)
            assert np.array_equal(engine.mul(b, a), want), (nb, na)
        a = rng.integers(0, 1 << 32, N // 2, dtype=np.uint64).astype(np.uint32)
        want = np.zeros(N, dtype=np.uint32)
        r = oracle.gmp_mul(a, a)
        want[:len(r)] = r
        assert np.array_equal(engine.sqr(a), want)
    finally:
        engine.set_plan(log_n, [])
    assert engine.device_errors() == 0
