"""Generate tests/golden/negacyclic_ref.json from the REFERENCE's own CPU
negacyclic multiply.

Run here, where the reference checkout exists:

    python tests/golden/make_negacyclic_golden.py

oracle/build.py compiles polymul_ntt_negacyclic
(ntt/ref/ntt_polymul_negacyclic.c:178-213) by path with
oracle/ref_negacyclic_shim.c into oracle/_ref/libref_nega.so. For each case
the inputs are f_i = splitmix64(seed_f, i) mod q and g_i likewise (the
counter form of cryptography_gb300/synth.py), and the record keeps the
sha256 of c = f * g mod (X^n + 1) mod q as little-endian uint64 words, with
its first and last words. The cases: the reference's own self-test
parameters (ML-DSA, n = 256, psi = 1753, ntt_polymul_negacyclic.c:391-396)
and NTT primes of the reference's modulus table (ntt/ref/ntt_moduli.h:265-279)
with psi = g^((q - 1) / 2n) from the table's primitive root g.
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from cryptography_gb300 import synth  # noqa: E402
from oracle import build  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "negacyclic_ref.json")

# (label, n, q, primitive root g of q or None, explicit psi or None)
CASES = [
    ("ML-DSA", 256, 8380417, None, 1753),
    ("FALCON", 32, 12289, 11, None),
    ("FHE-RNS", 4096, 2013265921, 31, None),
    ("CRT-mid", 16384, 469762049, 3, None),
]


def inputs(n, q, seed):
    return (synth.splitmix64(seed, 0, n) % np.uint64(q)).astype(np.uint64)


def main():
    so = build.build_ref_negacyclic()
    if so is None:
        sys.exit("reference checkout not found")
    R = ctypes.CDLL(so)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    R.ref_negacyclic_mul.restype = ctypes.c_int
    R.ref_negacyclic_mul.argtypes = [u64p, u64p, u64p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
    out = {}
    for k, (label, n, q, gen, psi) in enumerate(CASES):
        if psi is None:
            psi = pow(gen, (q - 1) // (2 * n), q)
        assert pow(psi, n, q) == q - 1, label   # primitive 2n-th root of unity
        sf, sg = 0x4E4701 + 2 * k, 0x4E4702 + 2 * k
        f, g = inputs(n, q, sf), inputs(n, q, sg)
        c = np.zeros(n, dtype=np.uint64)
        rc = R.ref_negacyclic_mul(f.ctypes.data_as(u64p), g.ctypes.data_as(u64p), c.ctypes.data_as(u64p), n, q, psi)
        assert rc == 0, label
        out[label] = {"n": n, "q": q, "psi": psi, "seed_f": sf, "seed_g": sg,
                      "sha256": hashlib.sha256(c.astype("<u8").tobytes()).hexdigest(),
                      "head": [int(v) for v in c[:8]], "tail": [int(v) for v in c[-8:]]}
    with open(OUT, "w") as fh:
        json.dump({"source": "ntt/ref/ntt_polymul_negacyclic.c:178-213 (polymul_ntt_negacyclic), built by path",
                   "cases": out}, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
