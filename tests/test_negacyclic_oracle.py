"""The negacyclic oracle against its definition (CPU): schoolbook sums with
the wrap-around sign, and the identity x * X = shift with the top
coefficient negated."""
import numpy as np

import oracle


def _schoolbook(f, g):
    n = len(f)
    c = [0] * n
    for i in range(n):
        for j in range(n):
            k = i + j
            if k < n:
                c[k] += int(f[i]) * int(g[j])
            else:
                c[k - n] -= int(f[i]) * int(g[j])
    return c


def test_negacyclic_oracle_matches_schoolbook():
    rng = np.random.default_rng(4)
    for n in (1, 2, 8, 32, 64):
        f = rng.integers(0, 1 << 64, n, dtype=np.uint64)
        g = rng.integers(0, 1 << 64, n, dtype=np.uint64)
        assert oracle.negacyclic_mul(f, g) == _schoolbook(f, g), n
    top = np.full(32, (1 << 64) - 1, dtype=np.uint64)
    assert oracle.negacyclic_mul(top, top) == _schoolbook(top, top)


def test_negacyclic_oracle_multiply_by_x():
    rng = np.random.default_rng(5)
    n = 128
    f = rng.integers(0, 1 << 64, n, dtype=np.uint64)
    x = np.zeros(n, dtype=np.uint64)
    x[1] = 1
    want = [-int(f[n - 1])] + [int(v) for v in f[:-1]]
    assert oracle.negacyclic_mul(f, x) == want
