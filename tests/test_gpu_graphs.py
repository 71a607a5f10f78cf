"""Batched waves replayed as CUDA graphs: a wave shape met a second time is
captured and replayed. Replays with fresh operands of other lengths in the
same bucket (other carry-tile counts, so the captured upper-bound carry grid
leaves surplus tiles) must give the same products as single multiplies and
the oracle; a plan change drops the captured graphs and the next waves use
the new plan."""
import numpy as np
import pytest

import oracle
from test_gpu_batch import _run_batch

pytestmark = pytest.mark.gpu


def _batch(rng, count, lo, hi):
    A, B = [], []
    for _ in range(count):
        na = int(rng.integers(lo, hi))
        nb = int(rng.integers(lo, hi))
        A.append(rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32))
        B.append(rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32))
    return A, B


def _check(engine, A, B, got, oracle_every=5):
    for i, (a, b, c) in enumerate(zip(A, B, got)):
        assert np.array_equal(c, engine.mul(a, b)), i
    for i in range(0, len(A), oracle_every):
        want = np.zeros(len(A[i]) + len(B[i]), dtype=np.uint32)
        r = oracle.mul(A[i], B[i])
        want[:len(r)] = r
        assert np.array_equal(got[i], want), i


def test_replayed_waves_match_single_products(engine):
    rng = np.random.default_rng(2024)
    before = engine.wave_graphs()
    # 24 products of 2^15-coefficient transforms (operands 4097 .. 16384
    # limbs) per call: the first call launches directly, the second captures,
    # the rest replay with other operand lengths
    for rep in range(5):
        A, B = _batch(rng, 24, 4097, 8193)
        _check(engine, A, B, _run_batch(engine, A, B))
    assert engine.wave_graphs() > before
    assert engine.device_errors() == 0


def test_plan_change_drops_graphs(engine):
    rng = np.random.default_rng(77)
    L = 14
    A, B = _batch(rng, 16, 2049, 4097)
    for _ in range(3):
        _run_batch(engine, A, B)
    assert engine.wave_graphs() > 0
    old = engine.plan(L)
    try:
        engine.set_plan(L, [5, 9] if old != [5, 9] else [7, 7])
        assert engine.wave_graphs() == 0
        for _ in range(3):
            A, B = _batch(rng, 16, 2049, 4097)
            _check(engine, A, B, _run_batch(engine, A, B), oracle_every=4)
    finally:
        engine.set_plan(L, [])
    assert engine.device_errors() == 0


def test_mixed_bucket_batches_replay(engine):
    # several buckets per call, each a different wave shape, repeated
    rng = np.random.default_rng(5)
    for _ in range(4):
        A, B = [], []
        for lo, hi, k in [(1, 200, 50), (600, 1000, 12), (3000, 4000, 9), (20000, 30000, 3)]:
            a, b = _batch(rng, k, lo, hi)
            A += a
            B += b
        _check(engine, A, B, _run_batch(engine, A, B), oracle_every=7)
    assert engine.device_errors() == 0
