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


def _fixture():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "negacyclic_ref.json")
    with open(path) as fh:
        return json.load(fh)["cases"]


def _inputs(n, q, seed):
    from cryptography_gb300 import synth
    return (synth.splitmix64(seed, 0, n) % np.uint64(q)).astype(np.uint64)


def test_negacyclic_oracle_matches_reference_fixture():
    # the definition-based oracle, reduced mod q, equals the reference's own
    # CPU negacyclic multiply (polymul_ntt_negacyclic,
    # ntt/ref/ntt_polymul_negacyclic.c:178-213) on the recorded cases
    import hashlib
    for label, c in _fixture().items():
        n, q = c["n"], c["q"]
        f, g = _inputs(n, q, c["seed_f"]), _inputs(n, q, c["seed_g"])
        got = np.array([v % q for v in oracle.negacyclic_mul(f, g)], dtype=np.uint64)
        assert [int(v) for v in got[:8]] == c["head"], label
        assert hashlib.sha256(got.astype("<u8").tobytes()).hexdigest() == c["sha256"], label


def test_reference_negacyclic_reproduces_fixture():
    # where the reference checkout exists, its multiply (built by path)
    # still gives the recorded outputs
    import ctypes
    import hashlib
    import pytest
    from oracle import build
    so = build.build_ref_negacyclic()
    if so is None:
        pytest.skip("reference checkout not present")
    R = ctypes.CDLL(so)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    R.ref_negacyclic_mul.restype = ctypes.c_int
    R.ref_negacyclic_mul.argtypes = [u64p, u64p, u64p] + [ctypes.c_uint64] * 3
    for label, c in _fixture().items():
        n, q = c["n"], c["q"]
        f, g = _inputs(n, q, c["seed_f"]), _inputs(n, q, c["seed_g"])
        out = np.zeros(n, dtype=np.uint64)
        assert R.ref_negacyclic_mul(f.ctypes.data_as(u64p), g.ctypes.data_as(u64p), out.ctypes.data_as(u64p),
                                    n, q, c["psi"]) == 0
        assert hashlib.sha256(out.astype("<u8").tobytes()).hexdigest() == c["sha256"], label
