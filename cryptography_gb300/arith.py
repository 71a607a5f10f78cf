"""Host mirror of the reference's arith layer above the multiply and of its
compute_e application (cecoppola/cryptography ``ntt/lib/arith/newton.h``,
``ntt/lib/arith/base_convert.h``, ``ntt/app/compute_e/binary_split.h`` and
``main.c``), on Python integers. Every call goes through libgbntt.so; all
products run on the GPU engine. The engine must be initialised
(``engine.init``) except for ``compute_e``, which sizes it itself when it is
not.
"""
import ctypes
import threading

import numpy as np

from . import engine

_u32p = ctypes.POINTER(ctypes.c_uint32)


def _limbs(v):
    if v < 0:
        raise ValueError("negative operand")
    n = max(1, (v.bit_length() + 31) // 32)
    return np.frombuffer(v.to_bytes(4 * n, "little"), dtype=np.uint32).copy()


def _int(a, n):
    return int.from_bytes(np.ascontiguousarray(a[:n], dtype=np.uint32).tobytes(), "little") if n else 0


def _out(n):
    return np.zeros(max(1, n), dtype=np.uint32)


def split_terms_needed(n_digits):
    """Series terms for n_digits digits (binary_split.c:96-108)."""
    return int(engine.lib().gbntt_split_terms_needed(int(n_digits)))


def e_required_log(digits):
    r = int(engine.lib().gbntt_e_required_log(int(digits)))
    if r < 0:
        engine._check(-r)
    return r


def binary_split(a, b):
    """(P, B) of the term range [a, b) (binary_split.c:26-86)."""
    # B = (b-1)!/(a-1)! has at most (b - a) * 32 bits; P < 2 B
    cap = max(2, (max(0, b - a)) + 4)
    p, q = _out(cap), _out(cap)
    np_, nq = ctypes.c_size_t(0), ctypes.c_size_t(0)
    engine._check(engine.lib().gbntt_binary_split(a, b, p.ctypes.data_as(_u32p), cap, ctypes.byref(np_),
                                                  q.ctypes.data_as(_u32p), cap, ctypes.byref(nq)))
    return _int(p, np_.value), _int(q, nq.value)


def newton_reciprocal(q):
    """floor(2^(2 bits(q)) / q) (newton.h:23)."""
    a = _limbs(q)
    cap = len(a) + 2
    x = _out(cap)
    n = ctypes.c_size_t(0)
    engine._check(engine.lib().gbntt_newton_reciprocal_u32(x.ctypes.data_as(_u32p), cap, ctypes.byref(n),
                                                           a.ctypes.data_as(_u32p), len(a)))
    return _int(x, n.value)


def div_newton(n, d):
    """(n // d, n % d) (newton.h:28)."""
    a, b = _limbs(n), _limbs(d)
    cq, cr = len(a) + 1, len(b) + 1
    q, r = _out(cq), _out(cr)
    nq, nr = ctypes.c_size_t(0), ctypes.c_size_t(0)
    engine._check(engine.lib().gbntt_div_newton_u32(q.ctypes.data_as(_u32p), cq, ctypes.byref(nq),
                                                    r.ctypes.data_as(_u32p), cr, ctypes.byref(nr),
                                                    a.ctypes.data_as(_u32p), len(a), b.ctypes.data_as(_u32p),
                                                    len(b)))
    return _int(q, nq.value), _int(r, nr.value)


def pow10_exact(e):
    """10^e (base_convert.h:32)."""
    cap = int(e * 3.3219280948873623 / 32) + 3
    x = _out(cap)
    n = ctypes.c_size_t(0)
    engine._check(engine.lib().gbntt_pow10_u32(x.ctypes.data_as(_u32p), cap, ctypes.byref(n), int(e)))
    return _int(x, n.value)


def to_decimal(v):
    """Decimal string of v (base_convert.h:24)."""
    a = _limbs(v)
    cap = int(len(a) * 32 * 0.30103) + 4
    buf = ctypes.create_string_buffer(cap)
    n = ctypes.c_size_t(0)
    engine._check(engine.lib().gbntt_to_decimal_u32(buf, cap, ctypes.byref(n), a.ctypes.data_as(_u32p), len(a)))
    return str(memoryview(buf)[:n.value], "ascii")


_e_buf = threading.local()   # per-thread output buffer reused across calls (a fresh 10^8-byte buffer costs a zero fill)


def e_buffer(digits):
    """A host buffer of at least digits + 2 bytes for gbntt_compute_e, kept
    between calls of the calling thread (threads do not share it)."""
    buf = getattr(_e_buf, "buf", None)
    if buf is None or len(buf) < int(digits) + 2:
        buf = _e_buf.buf = ctypes.create_string_buffer(int(digits) + 2)
    return buf


def compute_e_raw(digits, buf):
    """gbntt_compute_e into buf (from e_buffer); returns the 5 phase wall
    times (tree, numerator x 10^(D-1), division, decimal, total)."""
    ph = (ctypes.c_double * 5)()
    engine._check(engine.lib().gbntt_compute_e(int(digits), buf, len(buf), ph))
    return list(ph)


def compute_e(digits, phases=False):
    """"2.718..." with `digits` significant digits, as the reference's
    compute_e prints it after "e = " (main.c:340-345). With phases=True also
    returns the wall seconds (tree, numerator x 10^(D-1), division, decimal,
    total)."""
    buf = e_buffer(digits)
    ph = compute_e_raw(digits, buf)
    s = str(memoryview(buf)[:int(digits) + 1], "ascii")
    return (s, ph) if phases else s