"""The engine's largest transform (2^30 points: two 2^29-limb operands, 2 GiB
each). With two primes this needs p3's full 2-adicity (30) and the CRT
modulus q0 p3 ~ 2^95.6 above the largest coefficient, min(n_a, n_b)
(2^32 - 1)^2 < 2^93. Checked through size-independent properties (low limbs
against GMP, the whole integer modulo 62-bit moduli) and, for all-ones
operands (every coefficient at its maximum), against the closed form
(2^k - 1)^2 = 2^2k - 2^(k+1) + 1."""
import numpy as np
import pytest

import oracle
from cryptography_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def max_engine(built_lib):
    import cryptography_gb300 as g
    prev = g.lib().gbntt_max_log() if g.is_ready() else 0
    g.teardown()
    g.init(30)
    yield g
    g.teardown()
    if prev:
        g.init(prev)


def _moduli():
    rng = np.random.default_rng(2030)
    return [(1 << 61) - 1] + [int(x) | (1 << 61) | 1 for x in rng.integers(1 << 60, 1 << 62, 2, dtype=np.uint64)]


def test_max_transform_random(max_engine):
    n = 1 << 29
    assert max_engine.transform_log(n, n) == 30
    a = synth.operand(n, 91)
    b = synth.operand(n, 92)
    c = max_engine.mul(a, b)
    assert len(c) == 2 * n and (c[-1] != 0 or c[-2] != 0)
    K = 1 << 20
    assert np.array_equal(c[:K], oracle.gmp_mul(a[:K], b[:K])[:K])
    for q in _moduli():
        assert oracle.mod_u32(c, q) == oracle.mod_u32(a, q) * oracle.mod_u32(b, q) % q, q
    assert max_engine.device_errors() == 0


def test_max_transform_largest_coefficients(max_engine):
    n = 1 << 29
    a = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
    c = max_engine.sqr(a)
    assert c[0] == 1 and not c[1:n].any() and c[n] == 0xFFFFFFFE and (c[n + 1:] == 0xFFFFFFFF).all()
    assert max_engine.device_errors() == 0
