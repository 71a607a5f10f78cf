"""Full-size product (two 2^28-limb operands, transform length 2^29).

The multiply of the benchmark's operands (seeds 1 and 2) is compared limb
for limb with GMP mpz_mul of the same operands (about two minutes of one
host core, run in a thread while the GPU works), the shape of the
reference's oracle test (ntt/app/compute_e/test_gmp_oracle.c:70-76). Every
full-size product is also checked through size-independent properties:
  * the device Garner check reports no error (two primes: every
    coefficient below N 2^64; three primes: the third mixed-radix digit
    is 0);
  * the product agrees with the operands modulo several random 62-bit
    moduli (a checksum of the whole integer);
  * the low 2^20 limbs equal the low limbs of the GMP product of the low
    2^20 limbs of each operand (exact, limb for limb);
  * the limb count is exactly 2 n (both top bits set);
  * squaring and the packed (64-bit coefficient) form satisfy the same
    checks.
"""
import threading

import numpy as np
import pytest

import oracle
from cryptography_gb300 import synth

@pytest.fixture(scope="module")
def big_engine(built_lib):
    import cryptography_gb300 as g
    prev = g.lib().gbntt_max_log() if g.is_ready() else 0
    g.teardown()
    g.init(29)
    yield g
    g.teardown()
    if prev:
        g.init(prev)


def _moduli():
    rng = np.random.default_rng(2026)
    return [(1 << 61) - 1] + [int(x) | (1 << 61) | 1 for x in rng.integers(1 << 60, 1 << 62, 2, dtype=np.uint64)]


def _check_product(a, b, c):
    n = len(a)
    assert len(c) == len(a) + len(b)
    assert c[-1] != 0 or c[-2] != 0
    K = 1 << 20
    low = oracle.gmp_mul(a[:K], b[:K])
    assert np.array_equal(c[:K], low[:K])
    for q in _moduli():
        assert oracle.mod_u32(c, q) == oracle.mod_u32(a, q) * oracle.mod_u32(b, q) % q, q
    return n


@pytest.mark.gpu
@pytest.mark.slow
def test_full_size_multiply_every_limb_vs_gmp(big_engine):
    if not oracle.gmp_available():
        pytest.skip("libgmp.so.10 not available")
    n = 1 << 28
    a = synth.operand(n, 1)
    b = synth.operand(n, 2)
    ref = {}
    t = threading.Thread(target=lambda: ref.setdefault("c", oracle.gmp_mul(a, b)))
    t.start()                         # GMP on one host core while the GPU multiplies
    c = big_engine.mul(a, b)          # host path: raises on any device error flag
    _check_product(a, b, c)
    assert big_engine.device_errors() == 0
    t.join()
    want = ref["c"]
    assert len(want) == 2 * n
    diff = np.flatnonzero(c != want)
    assert diff.size == 0, "first differing limb %d of %d" % (int(diff[0]), diff.size)


@pytest.mark.gpu
def test_full_size_square(big_engine):
    n = 1 << 28
    a = synth.operand(n, 3)
    c = big_engine.sqr(a)
    _check_product(a, a, c)


@pytest.mark.gpu
def test_full_size_packed_multiply(big_engine):
    # the same 2^28 x 2^28 32-bit-limb integers as 2^27 x 2^27 64-bit limbs,
    # one coefficient per 64-bit limb (transform length 2^28)
    n = 1 << 28
    a = synth.operand(n, 5)
    b = synth.operand(n, 6)
    c = big_engine.mul64(a.view(np.uint64), b.view(np.uint64)).view(np.uint32)
    _check_product(a, b, c)
    assert big_engine.device_errors() == 0


def test_checksum_detects_corruption():
    # the property check itself is not vacuous: one flipped limb fails it
    # (planted on the CPU, in a copy of an oracle product)
    a = synth.operand(5000, 7)
    b = synth.operand(4000, 8)
    c = np.zeros(9000, dtype=np.uint32)
    r = oracle.mul(a, b)
    c[:len(r)] = r
    c[1234] ^= 1 << 17
    q = _moduli()[1]
    assert oracle.mod_u32(c, q) != oracle.mod_u32(a, q) * oracle.mod_u32(b, q) % q
