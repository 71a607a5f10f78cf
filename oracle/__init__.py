"""CPU oracle for the CRT-NTT multiply — TEST INFRASTRUCTURE ONLY.

The oracle restates the reference's CPU path (see the header of
``crt_ntt_oracle.c`` for the file:line map) and wraps GMP ``mpz_mul``
(ground truth) and, when the reference checkout is present, the reference's
own compiled host functions (``oracle/_ref``). Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
this package; the product never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)

PRIMES = (0xFFFFFFFF00000001, 0xFFFFFFFC00000001, 0xFFFFFF0000000001)
GENERATORS = (7, 10, 19)

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.oracle_reduce.restype = ctypes.c_uint64
        L.oracle_reduce.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]
        for name in ("oracle_mulmod", "oracle_addmod", "oracle_submod", "oracle_powmod"):
            f = getattr(L, name)
            f.restype = ctypes.c_uint64
            f.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_root.restype = ctypes.c_uint64
        L.oracle_root.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_ntt.restype = None
        L.oracle_ntt.argtypes = [ctypes.c_int, _u64p, ctypes.c_int, ctypes.c_int]
        L.oracle_garner3.restype = None
        L.oracle_garner3.argtypes = [ctypes.c_uint64] * 3 + [_u64p]
        L.oracle_gather_u32.restype = ctypes.c_long
        L.oracle_gather_u32.argtypes = [_u64p, ctypes.c_long, _u32p, ctypes.c_long]
        for name in ("oracle_mul_u32", "oracle_schoolbook_u32", "oracle_gmp_mul_u32"):
            f = getattr(L, name)
            f.restype = ctypes.c_long
            f.argtypes = [_u32p, ctypes.c_long, _u32p, ctypes.c_long, _u32p]
        L.oracle_mod_u32.restype = ctypes.c_uint64
        L.oracle_mod_u32.argtypes = [_u32p, ctypes.c_long, ctypes.c_uint64]
        L.oracle_mod_u32_par.restype = ctypes.c_uint64
        L.oracle_mod_u32_par.argtypes = [_u32p, ctypes.c_long, ctypes.c_uint64]
        L.oracle_gmp_available.restype = ctypes.c_int
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_threads.restype = None
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def ref():
    """The reference's own host code (compiled by path), or None."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None:
            return None
        R = ctypes.CDLL(path)
        R.ref_reduce.restype = ctypes.c_uint64
        R.ref_reduce.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]
        for name in ("ref_mulmod", "ref_addmod", "ref_submod", "ref_shoup_mul"):
            f = getattr(R, name)
            f.restype = ctypes.c_uint64
            f.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64]
        R.ref_prime.restype = ctypes.c_uint64
        R.ref_prime.argtypes = [ctypes.c_int]
        R.ref_prim_root.restype = ctypes.c_uint64
        R.ref_prim_root.argtypes = [ctypes.c_int]
        R.ref_garner4.restype = None
        R.ref_garner4.argtypes = [_u64p] * 5 + [ctypes.c_int]
        R.ref_scatter.restype = None
        R.ref_scatter.argtypes = [_u64p, ctypes.c_int, _u64p, ctypes.c_int, ctypes.c_int]
        R.ref_gather.restype = ctypes.c_int
        R.ref_gather.argtypes = [_u64p, ctypes.c_int, _u64p, ctypes.c_int]
        _ref = R
    return _ref


def _p32(a):
    return a.ctypes.data_as(_u32p)


def _p64(a):
    return a.ctypes.data_as(_u64p)


def _as_u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def mul(a, b):
    """CPU CRT-NTT product of two uint32 limb vectors (trimmed)."""
    a, b = _as_u32(a), _as_u32(b)
    c = np.zeros(len(a) + len(b), dtype=np.uint32)
    n = lib().oracle_mul_u32(_p32(a), len(a), _p32(b) if b is not a else _p32(a), len(b), _p32(c))
    return c[:n]


def square(a):
    a = _as_u32(a)
    c = np.zeros(2 * len(a), dtype=np.uint32)
    n = lib().oracle_mul_u32(_p32(a), len(a), _p32(a), len(a), _p32(c))
    return c[:n]


def schoolbook(a, b):
    a, b = _as_u32(a), _as_u32(b)
    c = np.zeros(len(a) + len(b), dtype=np.uint32)
    n = lib().oracle_schoolbook_u32(_p32(a), len(a), _p32(b), len(b), _p32(c))
    return c[:n]


def gmp_available():
    return bool(lib().oracle_gmp_available())


def gmp_mul(a, b):
    a, b = _as_u32(a), _as_u32(b)
    c = np.zeros(len(a) + len(b), dtype=np.uint32)
    n = lib().oracle_gmp_mul_u32(_p32(a), len(a), _p32(b), len(b), _p32(c))
    if n < 0:
        raise RuntimeError("libgmp.so.10 not available")
    return c[:n]


def ntt(prime_index, x, inverse=False):
    """Natural-order NTT (unscaled in the inverse direction)."""
    x = np.array(x, dtype=np.uint64, copy=True)
    log_n = int(len(x)).bit_length() - 1
    assert 1 << log_n == len(x)
    lib().oracle_ntt(prime_index, _p64(x), log_n, 1 if inverse else 0)
    return x


def root(prime_index, log_n, inverse=False):
    return int(lib().oracle_root(prime_index, log_n, 1 if inverse else 0))


def garner3(r0, r1, r2):
    out = (ctypes.c_uint64 * 4)()
    lib().oracle_garner3(r0, r1, r2, out)
    return sum(int(out[i]) << (64 * i) for i in range(4))


def gather_u32(coeff_words, out_cap):
    """coeff_words: (n, 4) uint64 little-endian words per coefficient."""
    cw = np.ascontiguousarray(coeff_words, dtype=np.uint64).reshape(-1)
    out = np.zeros(out_cap, dtype=np.uint32)
    n = lib().oracle_gather_u32(_p64(cw), len(cw) // 4, _p32(out), out_cap)
    return out[:n]


def mod_u32(a, q):
    """Value of the limb vector modulo q (q < 2^63), OpenMP-parallel."""
    a = _as_u32(a)
    return int(lib().oracle_mod_u32_par(_p32(a), len(a), q))


def to_int(limbs):
    """Python int from little-endian uint32 limbs."""
    return int.from_bytes(np.ascontiguousarray(limbs, dtype="<u4").tobytes(), "little")


def from_int(v, n=None):
    nb = max(1, (v.bit_length() + 31) // 32) if n is None else n
    return np.frombuffer(v.to_bytes(4 * nb, "little"), dtype="<u4").astype(np.uint32)


def num_threads():
    return int(lib().oracle_num_threads())


def set_threads(n):
    """OpenMP thread count of the oracle's parallel regions from now on."""
    lib().oracle_set_threads(int(n))


def negacyclic_mul(f, g):
    """Negacyclic convolution mod X^N + 1 of two length-N sequences of
    unsigned 64-bit coefficients, as exact Python ints (signed):
    c_k = sum_{i+j=k} f_i g_j - sum_{i+j=k+N} f_i g_j. This is the product
    the reference's crt_ntt negacyclic pipeline computes
    (ntt/lib/main.hip:557-684), stated by its definition; evaluated here by
    Kronecker substitution (one big-integer product of the two sequences
    packed into byte-aligned slots wide enough for every full-product
    coefficient, < N 2^128)."""
    f = np.ascontiguousarray(f, dtype=np.uint64)
    g = np.ascontiguousarray(g, dtype=np.uint64)
    n = len(f)
    if len(g) != n:
        raise ValueError("f and g need the same length")
    if n == 0:
        return []
    slot = (128 + n.bit_length() + 8) // 8   # bytes per slot

    def pack(x):
        buf = np.zeros((n, slot), dtype=np.uint8)
        buf[:, :8] = x.view(np.uint8).reshape(n, 8)
        return int.from_bytes(buf.tobytes(), "little")

    prod = pack(f) * pack(g)
    raw = np.frombuffer(prod.to_bytes(2 * n * slot, "little"), dtype=np.uint8).reshape(2 * n, slot)
    d = [int.from_bytes(raw[k].tobytes(), "little") for k in range(2 * n)]
    return [d[k] - d[k + n] for k in range(n)]
