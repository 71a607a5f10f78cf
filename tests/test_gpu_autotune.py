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
