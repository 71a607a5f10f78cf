"""CPU tests: the oracle restatement pinned against the reference's own code
(golden vectors from tests/golden/make_golden.py), GMP and Python integers.
Mirrors the reference's host suites: test_reduce.c / test_modops.hip
(modular ops), test_garner.cpp (Garner), test_arith.c:457-523 (gather KATs),
test_e2e_oracle.c (whole CRT-NTT method on the CPU) and test_ntt_kernel.hip
KA1-KA6 (transform known answers)."""
import hashlib

import numpy as np
import pytest

import oracle
from cryptography_gb300 import synth


def test_primes_and_generators(golden):
    for i, m in enumerate(golden["modops"]):
        assert m["p"] == oracle.PRIMES[i]
        assert m["prim_root"] == oracle.GENERATORS[i]
        p = m["p"]
        # generator is a non-residue, so g^((p-1)/N) has order exactly N
        assert pow(m["prim_root"], (p - 1) // 2, p) == p - 1
        w = oracle.root(i, 30)
        assert pow(w, 1 << 30, p) == 1 and pow(w, 1 << 29, p) == p - 1


@pytest.mark.parametrize("section", ["reduce", "mulmod", "addmod", "submod"])
def test_modops_match_reference(golden, section):
    L = oracle.lib()
    fn = {"reduce": L.oracle_reduce, "mulmod": L.oracle_mulmod, "addmod": L.oracle_addmod,
          "submod": L.oracle_submod}[section]
    n = 0
    for i, m in enumerate(golden["modops"]):
        for x, y, want in m[section]:
            assert fn(i, x, y) == want, (section, i, x, y)
            n += 1
    assert n > 500


def test_shoup_equals_mulmod(golden):
    # the reference's Shoup twiddle multiply and this engine's multiply agree
    for i, m in enumerate(golden["modops"]):
        for t, w, want in m["shoup_mul"]:
            assert oracle.lib().oracle_mulmod(i, t, w) == want


def test_modops_random_vs_python():
    rng = np.random.default_rng(5)
    for i, p in enumerate(oracle.PRIMES):
        for _ in range(2000):
            a, b = (int(x) % p for x in rng.integers(0, 1 << 64, 2, dtype=np.uint64))
            assert oracle.lib().oracle_mulmod(i, a, b) == a * b % p
            assert oracle.lib().oracle_addmod(i, a, b) == (a + b) % p
            assert oracle.lib().oracle_submod(i, a, b) == (a - b) % p
            hi, lo = int(rng.integers(0, 1 << 63)) % p, int(rng.integers(0, 1 << 64, dtype=np.uint64))
            assert oracle.lib().oracle_reduce(i, lo, hi) == ((hi << 64) | lo) % p


def test_scatter_matches_reference(golden):
    # bigint_scatter of a 64-bit limb = limb mod p; a 32-bit limb is its own residue
    for s in golden["scatter"]:
        p = oracle.PRIMES[s["prime_index"]]
        want = [x % p for x in s["limbs"]] + [0] * (20 - len(s["limbs"]))
        assert s["coeffs"] == want


def _words32(cw64):
    """U256 coefficients at 64-bit offsets -> coefficients at 32-bit offsets
    (odd positions zero), as (n, 4) uint64 words."""
    out = np.zeros((2 * len(cw64), 4), dtype=np.uint64)
    out[0::2] = np.array(cw64, dtype=np.uint64)
    return out


def test_gather_matches_reference(golden):
    for g in golden["gather"]:
        want = sum(int(v) << (64 * k) for k, v in enumerate(g["limbs"]))
        got = oracle.to_int(oracle.gather_u32(_words32(g["coeffs"]), 2 * len(g["coeffs"]) + 16))
        assert got == want


def test_gather_kats():
    # the gather known answers of ntt/lib/arith/test_arith.c:457-523, restated
    # for 32-bit limb offsets
    def g1(w):
        return oracle.to_int(oracle.gather_u32(np.array([w], dtype=np.uint64), 12))
    assert g1([42, 0, 0, 0]) == 42
    assert g1([0, 0, 1, 0]) == 340282366920938463463374607431768211456
    assert g1([0, 0, 0, 1]) == 6277101735386680763835789423207666416102355444464034512896
    assert g1([1, 1, 1, 1]) == 1 + (1 << 64) + (1 << 128) + (1 << 192)
    A = (1 << 300) + 123456789
    limbs = oracle.from_int(A)
    cw = np.zeros((len(limbs), 4), dtype=np.uint64)
    cw[:, 0] = limbs
    assert oracle.to_int(oracle.gather_u32(cw, len(limbs) + 8)) == A


def _crt(rs, ps):
    M = 1
    for p in ps:
        M *= p
    x = 0
    for r, p in zip(rs, ps):
        Mi = M // p
        x += r * Mi * pow(Mi, -1, p)
    return x % M


def test_garner4_reference_is_crt(golden):
    # pins the reference's mixed-radix Garner method against Python CRT
    P = golden["garner4"]["primes"]
    for t, words in golden["garner4"]["cases"]:
        got = sum(int(w) << (64 * k) for k, w in enumerate(words))
        assert got == _crt(t, P)


def test_garner3_matches_crt():
    rng = np.random.default_rng(7)
    P = oracle.PRIMES
    cases = [(0, 0, 0), (1, 1, 1), (P[0] - 1, P[1] - 1, P[2] - 1)]
    cases += [tuple(int(rng.integers(0, 1 << 63)) * 2 % p for p in P) for _ in range(3000)]
    for r in cases:
        assert oracle.garner3(*r) == _crt(r, P)
    # known single-word vectors (test_garner.cpp check A)
    for x in (0, 5, 1 << 40, P[2] - 1):
        assert oracle.garner3(x, x, x) == x


def test_ntt_known_answers():
    # KA1..KA6 of ntt/app/compute_e/test_ntt_kernel.hip:13-26, all three primes
    for i, p in enumerate(oracle.PRIMES):
        for log_n in (1, 5, 10):
            n = 1 << log_n
            d0 = np.zeros(n, dtype=np.uint64); d0[0] = 1
            d1 = np.zeros(n, dtype=np.uint64); d1[1 % n] = 1
            X0 = oracle.ntt(i, d0)
            assert np.all(X0 == 1)                                         # KA1
            ninv = pow(n, -1, p)
            back = [int(v) * ninv % p for v in oracle.ntt(i, X0, inverse=True)]
            assert back == [int(v) for v in d0]                            # KA2
            w = oracle.root(i, log_n)
            X1 = oracle.ntt(i, d1)
            assert [int(v) for v in X1] == [pow(w, k, p) for k in range(n)]  # KA4
            prod = np.array([int(a) * int(b) % p for a, b in zip(X0, X1)], dtype=np.uint64)
            conv = [int(v) * ninv % p for v in oracle.ntt(i, prod, inverse=True)]
            assert conv == [int(v) for v in d1]                            # KA3
            geo = np.array([pow(w, k, p) for k in range(n)], dtype=np.uint64)
            back1 = [int(v) * ninv % p for v in oracle.ntt(i, geo, inverse=True)]
            assert back1 == [int(v) for v in d1]                           # KA5
            ones = np.ones(n, dtype=np.uint64)
            alt = np.array([1 if k % 2 == 0 else p - 1 for k in range(n)], dtype=np.uint64)
            had = [int(a) * int(b) % p for a, b in zip(ones, alt)]
            assert had == [int(v) for v in alt]                            # KA6


def test_ntt_matches_naive_dft():
    rng = np.random.default_rng(3)
    for i, p in enumerate(oracle.PRIMES):
        n = 64
        x = [int(v) % p for v in rng.integers(0, 1 << 64, n, dtype=np.uint64)]
        w = oracle.root(i, 6)
        want = [sum(x[j] * pow(w, j * k, p) for j in range(n)) % p for k in range(n)]
        assert [int(v) for v in oracle.ntt(i, np.array(x, dtype=np.uint64))] == want


SWEEP = [50, 65, 66, 80, 100, 127, 128, 129, 200, 256, 257, 400, 512, 513, 700, 1000, 1024, 1025, 1500, 2000,
         2048, 2049]   # size list of ntt/app/compute_e/test_polymul_sweep.hip:114-115


def test_oracle_products_vs_schoolbook_and_gmp():
    rng = np.random.default_rng(11)
    pairs = [(1, 1), (1, 7), (2, 2), (3, 5)] + [(SWEEP[i], SWEEP[j]) for i in range(len(SWEEP))
                                                  for j in range(len(SWEEP)) if (i + j) % 5 == 0]
    for na, nb in pairs:
        a = rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        c = oracle.mul(a, b)
        assert np.array_equal(c, oracle.schoolbook(a, b)), (na, nb)
        if oracle.gmp_available():
            assert np.array_equal(c, oracle.gmp_mul(a, b)), (na, nb)
        assert oracle.to_int(c) == oracle.to_int(a) * oracle.to_int(b)


def test_oracle_all_max_limbs():
    # all-0xFFFFFFFF operands: maximal coefficients and carry chains
    for n in (1, 31, 32, 33, 1000):
        a = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
        v = (1 << (32 * n)) - 1
        assert oracle.to_int(oracle.mul(a, a)) == v * v
        assert oracle.to_int(oracle.square(a)) == v * v


def test_golden_products_oracle(golden):
    for pr in golden["products"]:
        if pr["na"] + pr["nb"] > (1 << 18):
            continue
        a = synth.operand(pr["na"], pr["seed_a"])
        b = synth.operand(pr["nb"], pr["seed_b"])
        c = oracle.mul(a, b)
        full = np.zeros(pr["na"] + pr["nb"], dtype=np.uint32)
        full[:len(c)] = c
        assert hashlib.sha256(full.astype("<u4").tobytes()).hexdigest() == pr["sha256"]


def test_synth_operand_shape():
    a = synth.operand(1000, 42)
    assert a.dtype == np.uint32 and len(a) == 1000 and a[-1] >> 31 == 1
    b = synth.operand(1 << 20, 42, chunk=1 << 12)      # chunking does not change limbs
    assert np.array_equal(a[:-1], b[:999])
    assert not np.array_equal(a[:100], synth.operand(100, 43)[:100])


@pytest.mark.skipif(oracle.ref() is None, reason="reference checkout not present")
def test_oracle_vs_reference_random():
    R = oracle.ref()
    rng = np.random.default_rng(99)
    for bi, rp in enumerate((0, 2, 3)):
        for _ in range(3000):
            lo, hi = (int(x) for x in rng.integers(0, 1 << 64, 2, dtype=np.uint64))
            hi %= oracle.PRIMES[bi]
            assert oracle.lib().oracle_reduce(bi, lo, hi) == R.ref_reduce(rp, lo, hi)
