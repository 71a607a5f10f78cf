"""Generate tests/golden/golden.json from the REFERENCE's own host code.

Run here, where the reference checkout exists:

    python tests/golden/make_golden.py

It compiles the reference's primes.h / shoup.h / garner.hip / bigint.c by
path (oracle/build.py -> oracle/_ref/libref.so) and records their outputs on
seeded inputs, plus GMP products. The committed JSON then pins the oracle on
machines without the reference checkout.

Sections:
  modops   reduce_p*/mulmod/addmod/submod/shoup_mul of the reference
           (ntt/lib/primes.h:57-217, ntt/lib/shoup.h:69-112), primes P0, P2, P3
  scatter  bigint_scatter (ntt/lib/arith/bigint.c:286-294)
  gather   bigint_gather (ntt/lib/arith/bigint.c:333-397) on U256 coefficients
  garner4  the reference's 4-prime Garner (ntt/lib/garner.hip:105-173)
  products sha256 of GMP products of seeded synthetic operands
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cryptography_gb300 import synth  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
REF_PIDX = (0, 2, 3)   # reference prime index of this engine's primes 0, 1, 2
M64 = (1 << 64) - 1


def corner_values(p):
    return [0, 1, 2, p - 1, p - 2, p >> 1, (p + 1) >> 1, 1 << 32, (1 << 32) - 1, 1 << 63, M64, M64 - 1,
            p + 1 if p + 1 <= M64 else 0]


def main():
    R = oracle.ref()
    if R is None:
        sys.exit("reference checkout not found; golden vectors come from the reference's own code")
    rng = np.random.default_rng(20261203)
    gold = {"source": "reference host code compiled by path (oracle/ref_shim.cpp)", "modops": []}
    for bi, rp in enumerate(REF_PIDX):
        p = int(R.ref_prime(rp))
        vals = corner_values(p) + [int(x) for x in rng.integers(0, 1 << 63, 24, dtype=np.uint64) * 2 + 1]
        red = []
        for lo in vals:
            for hi in vals[:8]:
                if hi >= p:
                    continue
                red.append([lo, hi, int(R.ref_reduce(rp, lo, hi))])
        canon = [v % p for v in vals]
        mul = [[a, b, int(R.ref_mulmod(rp, a, b))] for a in canon for b in canon[:10]]
        add = [[a, b, int(R.ref_addmod(rp, a, b))] for a in canon for b in canon[:10]]
        sub = [[a, b, int(R.ref_submod(rp, a, b))] for a in canon for b in canon[:10]]
        shoup = [[a, b, int(R.ref_shoup_mul(rp, a, b))] for a in canon for b in canon[:6]]
        gold["modops"].append({"prime_index": bi, "reference_pidx": rp, "p": p, "prim_root": int(R.ref_prim_root(rp)),
                               "reduce": red, "mulmod": mul, "addmod": add, "submod": sub, "shoup_mul": shoup})

    # scatter: 64-bit limbs mod p, zero padded to n_coeffs
    sc = []
    for bi, rp in enumerate(REF_PIDX):
        limbs = np.array([0, 1, M64, M64 - 1, int(R.ref_prime(rp)), int(R.ref_prime(rp)) - 1] +
                         [int(x) for x in rng.integers(0, 1 << 64, 10, dtype=np.uint64)], dtype=np.uint64)
        coeffs = np.zeros(20, dtype=np.uint64)
        R.ref_scatter(limbs.ctypes.data_as(oracle._u64p), len(limbs), coeffs.ctypes.data_as(oracle._u64p), 20, rp)
        sc.append({"prime_index": bi, "limbs": [int(x) for x in limbs], "coeffs": [int(x) for x in coeffs]})
    gold["scatter"] = sc

    # gather: U256 coefficients (4 words) at 64-bit offsets -> 64-bit limbs
    ga = []
    cases = [[[42, 0, 0, 0]], [[0, 0, 1, 0]], [[0, 0, 0, 1]], [[1, 1, 1, 1]], [[M64, M64, M64, M64]] * 5]
    for _ in range(6):
        n = int(rng.integers(1, 12))
        cases.append([[int(x) for x in rng.integers(0, 1 << 64, 4, dtype=np.uint64)] for _ in range(n)])
    for cw in cases:
        arr = np.array(cw, dtype=np.uint64).reshape(-1)
        cap = len(cw) + 8
        out = np.zeros(cap, dtype=np.uint64)
        n = R.ref_gather(arr.ctypes.data_as(oracle._u64p), len(cw), out.ctypes.data_as(oracle._u64p), cap)
        ga.append({"coeffs": cw, "limbs": [int(x) for x in out[:n]]})
    gold["gather"] = ga

    # garner over the reference's 4 primes
    P = [int(R.ref_prime(i)) for i in range(4)]
    tuples = [[0, 0, 0, 0], [1, 1, 1, 1], [P[0] - 1, P[1] - 1, P[2] - 1, P[3] - 1], [12345, 12345, 12345, 12345]]
    for _ in range(40):
        tuples.append([int(rng.integers(0, P[i] // 2)) * 2 + int(rng.integers(0, 2)) for i in range(4)])
    cols = [np.array([t[i] for t in tuples], dtype=np.uint64) for i in range(4)]
    out = np.zeros(4 * len(tuples), dtype=np.uint64)
    R.ref_garner4(*(c.ctypes.data_as(oracle._u64p) for c in cols), out.ctypes.data_as(oracle._u64p), len(tuples))
    gold["garner4"] = {"primes": P, "cases": [[t, [int(x) for x in out[4 * i:4 * i + 4]]]
                                              for i, t in enumerate(tuples)]}

    # GMP products of seeded synthetic operands (sha256 of the limb bytes)
    prods = []
    for na, nb, sa, sb in [(1, 1, 1, 2), (5, 3, 3, 4), (64, 65, 5, 6), (1000, 999, 7, 8), (4096, 4096, 9, 10),
                           (1 << 16, 1 << 16, 11, 12), (1 << 18, 3, 13, 14), ((1 << 20), (1 << 20), 15, 16)]:
        a = synth.operand(na, sa)
        b = synth.operand(nb, sb)
        c = oracle.gmp_mul(a, b)
        full = np.zeros(na + nb, dtype=np.uint32)
        full[:len(c)] = c
        prods.append({"na": na, "nb": nb, "seed_a": sa, "seed_b": sb,
                      "sha256": hashlib.sha256(full.astype("<u4").tobytes()).hexdigest()})
    gold["products"] = prods
    with open(OUT, "w") as f:
        json.dump(gold, f, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
