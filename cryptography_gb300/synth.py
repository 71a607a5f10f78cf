"""Seeded synthetic operands.

Limb i of an operand is the low 32 bits of splitmix64 evaluated at
seed + (i + 1) * 0x9E3779B97F4A7C15 (the generator of the reference sweep,
ntt/app/compute_e/test_polymul_sweep.hip:29-34, in counter form so any limb
can be produced independently). The top limb is OR-ed with 2^31 so an
operand of n limbs has exactly n significant limbs (as test_gmp_oracle.c:70-71
forces the top bit of a 64-bit limb).
"""
import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, start, count):
    """splitmix64 outputs for counters start+1 .. start+count (uint64 array)."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + i * GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def operand(n, seed, chunk=1 << 24):
    """n uniform random 32-bit limbs with the top bit of the top limb set."""
    out = np.empty(n, dtype=np.uint32)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        out[s:s + m] = splitmix64(seed, s, m).astype(np.uint32)
    if n:
        out[n - 1] |= np.uint32(1 << 31)
    return out


def batched_sizes(pairs, seed, lo=10, hi=22):
    """Operand sizes of a batch of uneven products: log2(n) uniform in
    [lo, hi) per operand, drawn independently for the two operands of every
    pair from a seeded generator (limb counts, int64 arrays)."""
    rng = np.random.default_rng(seed)
    na = np.floor(2.0 ** rng.uniform(lo, hi, pairs)).astype(np.int64)
    nb = np.floor(2.0 ** rng.uniform(lo, hi, pairs)).astype(np.int64)
    return na, nb
