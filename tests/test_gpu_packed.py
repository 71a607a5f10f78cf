"""Packed mode (one 64-bit limb per NTT coefficient, the reference engine's
own granularity): products through the C ABI compared bit-for-bit with GMP
and the oracle. A 64-bit limb can exceed the primes (all of them are below
2^64), so all-ones limbs exercise the limb -> residue reduction."""
import json
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle
from cryptography_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rand64(rng, n):
    return rng.integers(0, 1 << 64, n, dtype=np.uint64)


def _want(a, b):
    c = oracle.gmp_mul(a.view(np.uint32), b.view(np.uint32))
    out = np.zeros(2 * (len(a) + len(b)), dtype=np.uint32)
    out[:len(c)] = c
    return out.view(np.uint64)


def test_packed_small_and_sweep(engine):
    rng = np.random.default_rng(21)
    sizes = [1, 2, 3, 16, 17, 31, 32, 33, 100, 511, 512, 513, 1000, 4097]
    for i, na in enumerate(sizes):
        for nb in sizes[i::3]:
            a, b = _rand64(rng, na), _rand64(rng, nb)
            assert np.array_equal(engine.mul64(a, b), _want(a, b)), (na, nb)
    assert engine.device_errors() == 0


@pytest.mark.parametrize("log_n", [5, 10, 11, 15, 20, 21, 23])
def test_packed_length_boundaries(engine, log_n):
    rng = np.random.default_rng(60 + log_n)
    N = 1 << log_n
    for need in (N, N - 1):
        na = need // 2 + 1
        nb = need + 1 - na
        a, b = _rand64(rng, na), _rand64(rng, nb)
        assert np.array_equal(engine.mul64(a, b), _want(a, b)), (log_n, na, nb)


def test_packed_limbs_above_primes(engine):
    # all-ones limbs exceed every prime: the decomposition must reduce them
    for n in (1, 7, 1000, 1 << 16):
        a = np.full(n, (1 << 64) - 1, dtype=np.uint64)
        v = (1 << (64 * n)) - 1
        got = engine.mul64(a, a)
        assert oracle.to_int(got.view(np.uint32)) == v * v, n
    P = oracle.PRIMES
    a = np.array([P[0], P[1], P[2], P[0] - 1, P[2] + 1, (1 << 63), 0, 5], dtype=np.uint64)
    b = a[::-1].copy()
    assert np.array_equal(engine.mul64(a, b), _want(a, b))
    assert engine.device_errors() == 0


def test_packed_square_and_equivalence(engine):
    rng = np.random.default_rng(22)
    for n in (1, 5, 3000, 1 << 17):
        a = _rand64(rng, n)
        got = engine.mul64(a, a)
        assert np.array_equal(got, _want(a, a)), n
        # same integers through the 32-bit coefficient path
        assert np.array_equal(engine.mul(a.view(np.uint32), a.view(np.uint32)), got.view(np.uint32))


def test_packed_2pow22(engine):
    a = synth.operand(1 << 23, 31).view(np.uint64)
    b = synth.operand(1 << 23, 32).view(np.uint64)
    assert np.array_equal(engine.mul64(a, b), _want(a, b))
    assert engine.device_errors() == 0


def test_bigint_api_packed_mode():
    body = textwrap.dedent("""
        import json, random, sys
        sys.path.insert(0, %r)
        import ctypes
        import cryptography_gb300 as g
        L = g.lib()
        L.ntt_mul_init_impl(20)
        rng = random.Random(3)
        ok = []
        for na, nb in [(1, 1), (3, 2), (1000, 77), (1 << 18, (1 << 18) - 3)]:
            x = rng.getrandbits(64 * na) | (1 << (64 * na - 1))
            y = rng.getrandbits(64 * nb) | (1 << (64 * nb - 1))
            a, b, c = g.bigint_from_int(x), g.bigint_from_int(y), g.bigint_alloc(2)
            L.ntt_bigint_mul(ctypes.byref(c), ctypes.byref(a), ctypes.byref(b))
            ok.append(g.bigint_to_int(c) == x * y)
        print(json.dumps([L.gbntt_coeff_bits(), ok]))
    """ % ROOT)
    env = dict(os.environ, GBNTT_COEFF_BITS="64")
    r = subprocess.run([sys.executable, "-c", body], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    bits, ok = json.loads(r.stdout.strip().splitlines()[-1])
    assert bits == 64 and all(ok)
