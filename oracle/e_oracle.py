"""CPU oracle of the reference's compute_e path — TEST INFRASTRUCTURE ONLY.

Plain-Python restatement (small cases) of:
  * split_terms_needed   ntt/app/compute_e/binary_split.c:96-108
  * binary_split         ntt/app/compute_e/binary_split.c:26-86
  * compute_e's result   ntt/app/compute_e/main.c:167-296 and :340-345:
    floor((B + P) 10^(D+20) / B), printed as d0 "." d1..d(D-1)
  * newton_reciprocal    ntt/lib/arith/newton.h:15-23 (the exact floor; the
    reference's may be one below, never above)
e_gmp_oracle.c restates the same path in C on GMP for large digit counts.
Pinned by tests/golden/e_digits.json (sha256 of the reference's own printed
digits, generated by tests/golden/make_e_golden.py from the reference's
compiled host compute_e). Only tests/ and bench.py's CPU legs use it.
"""
import ctypes
import math
import sys

from . import build as _build

_elib = None


def _e_lib():
    global _elib
    if _elib is None:
        L = ctypes.CDLL(_build.build_e_oracle())
        L.oracle_e_digits.argtypes = [ctypes.c_long, ctypes.c_char_p, ctypes.c_size_t,
                                      ctypes.POINTER(ctypes.c_double)]
        L.oracle_e_digits.restype = ctypes.c_int
        L.oracle_split_terms_needed.argtypes = [ctypes.c_long]
        L.oracle_split_terms_needed.restype = ctypes.c_long
        _elib = L
    return _elib


def gmp_e_string(digits):
    """(string, seconds): the same e string from e_gmp_oracle.c (GMP, one
    thread) — usable at 10^7..10^8 digits and as the CPU baseline."""
    buf = ctypes.create_string_buffer(int(digits) + 2)
    sec = ctypes.c_double(0)
    if _e_lib().oracle_e_digits(int(digits), buf, int(digits) + 2, ctypes.byref(sec)) != 0:
        raise RuntimeError("oracle_e_digits failed")
    return buf.raw[:int(digits) + 1].decode(), sec.value


def split_terms_needed(n_digits):
    target = n_digits * math.log(10.0)
    N = target / math.log(target)
    for _ in range(50):
        logN = math.log(N)
        if logN <= 1.0:
            N = target
            break
        N = target / (logN - 1.0)
    return int(N * 1.05) + 64


def binary_split(a, b):
    """(P, B) of [a, b): B = (b-1)!/(a-1)!, P/B = sum_{k=a}^{b-1} (a-1)!/k!."""
    if b <= a:
        return 0, 1
    if b - a == 1:
        return 1, a
    m = a + (b - a) // 2
    pl, bl = binary_split(a, m)
    pr, br = binary_split(m, b)
    return pl * br + pr, bl * br


def binary_split_seq(a, b):
    """Same P, B by folding term by term (P <- P k + 1, B <- B k)."""
    p, q = 0, 1
    for k in range(a, b):
        p = p * k + 1
        q *= k
    return p, q


def newton_reciprocal(q):
    return (1 << (2 * q.bit_length())) // q


def e_string(digits, guard=20):
    """The reference's printed e string for `digits` digits (Python ints)."""
    if hasattr(sys, "set_int_max_str_digits"):
        sys.set_int_max_str_digits(0)
    n_total = digits + guard
    K = split_terms_needed(n_total)
    P, B = binary_split(1, K + 1)
    result = (B + P) * 10 ** n_total // B
    dec = str(result)
    return dec[0] + "." + dec[1:digits]
