"""Bounded waits: a carry look-back that waits on a status word nothing
writes must give up within its iteration limit, report the error bit to the
host and leave the context usable (no fault, trap or hang is involved: the
wait simply runs out)."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ERR_LOOKBACK_TIMEOUT = 2


def test_lookback_wait_runs_out_and_reports(engine):
    flags, sec = ctypes.c_uint(0), ctypes.c_double(0)
    assert engine.lib().gbntt_debug_lookback_timeout(ctypes.byref(flags), ctypes.byref(sec)) == 0
    assert flags.value & ERR_LOOKBACK_TIMEOUT
    assert 0 < sec.value < 30
    # the flag was consumed and the engine still multiplies correctly
    assert engine.device_errors() == 0
    rng = np.random.default_rng(5)
    a = rng.integers(0, 1 << 32, 5000, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 1 << 32, 3000, dtype=np.uint64).astype(np.uint32)
    want = np.zeros(8000, dtype=np.uint32)
    r = oracle.mul(a, b)
    want[:len(r)] = r
    assert np.array_equal(engine.mul(a, b), want)
    assert engine.device_errors() == 0
