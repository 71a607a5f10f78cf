"""GPU tests of libgbntt112.so, the reference entry points for the
reference's LIMB_BITS=112 BigInt build (ntt/lib/arith/bigint.h:30-43:
16-byte limbs holding 112 bits, value = sum limbs[i] 2^(112 i)). Each case
runs in a child process, as tests/test_gpu_bigint.py does for the 64-bit
flavour: the engine is process-global and the guard paths exit the
process."""
import json
import os
import subprocess
import sys
import textwrap

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = textwrap.dedent("""
    import ctypes, json, os, random, sys
    sys.path.insert(0, %r)
    from cryptography_gb300 import build
    build.build()
    L = ctypes.CDLL(build.LIB112)
    libc = ctypes.CDLL(None)
    libc.malloc.restype = ctypes.c_void_p
    libc.malloc.argtypes = [ctypes.c_size_t]
    libc.free.argtypes = [ctypes.c_void_p]
    U64P = ctypes.POINTER(ctypes.c_uint64)
    class BigInt112(ctypes.Structure):
        _fields_ = [("limbs", U64P), ("n_limbs", ctypes.c_int), ("cap", ctypes.c_int), ("managed", ctypes.c_int)]
    L.bigint_alloc_managed.restype = BigInt112
    L.bigint_alloc_managed.argtypes = [ctypes.c_int]
    L.ntt_bigint_mul_checked.restype = ctypes.c_int
    L.ntt_get_gpu_dispatch_count.restype = ctypes.c_ulong
    M112 = (1 << 112) - 1
    def nlimbs(v):
        return (v.bit_length() + 111) // 112
    def set_int(b, v):
        n = nlimbs(v)
        assert n <= b.cap
        for i in range(b.cap):
            w = (v >> (112 * i)) & M112 if i < n else 0
            b.limbs[2 * i] = w & ((1 << 64) - 1)
            b.limbs[2 * i + 1] = w >> 64
        b.n_limbs = n
    def alloc(cap):
        p = libc.malloc(16 * max(cap, 1))
        ctypes.memset(p, 0, 16 * max(cap, 1))
        return BigInt112(ctypes.cast(p, U64P), 0, cap, 0)
    def from_int(v, cap=None):
        b = alloc(max(cap or 0, nlimbs(v), 1))
        set_int(b, v)
        return b
    def to_int(b):
        v = 0
        for i in range(b.n_limbs):
            w = b.limbs[2 * i] | (b.limbs[2 * i + 1] << 64)
            assert w <= M112
            v |= w << (112 * i)
        return v
    def tail_zero(b):
        return all(b.limbs[k] == 0 for k in range(2 * b.n_limbs, 2 * b.cap))
    def free(b):
        libc.free(ctypes.cast(b.limbs, ctypes.c_void_p))
    def rnd(rng, n):
        return rng.getrandbits(112 * n) | (1 << (112 * n - 1)) if n else 0
    B = ctypes.byref
""" % ROOT)


def run(body, env=None, timeout=600):
    e = dict(os.environ)
    e.pop("NTT_MAX_LOGN", None)
    if env:
        e.update(env)
    return subprocess.run([sys.executable, "-c", PRELUDE + textwrap.dedent(body)], capture_output=True, text=True,
                          timeout=timeout, env=e)


def test_limb112_products_match_python_ints():
    r = run("""
        L.ntt_mul_init_impl(20)
        rng = random.Random(5)
        out = []
        cases = [(1, 1), (2, 1), (33, 17), (1000, 999), (4096, 4096), (70000, 3), (1 << 17, (1 << 17) - 5)]
        for na, nb in cases:
            x, y = rnd(rng, na), rnd(rng, nb)
            a, b = from_int(x), from_int(y)
            c = alloc(1)                                  # too small: the library grows it
            L.ntt_bigint_mul(B(c), B(a), B(b))
            out.append([na, nb, to_int(c) == x * y, c.cap >= na + nb + 4, tail_zero(c),
                        c.n_limbs == nlimbs(x * y)])
            for v in (a, b, c):
                free(v)
        big = (1 << (112 * 3000)) - 1                    # every limb 2^112 - 1
        a, b, c = from_int(big), from_int(big), alloc(8)
        L.ntt_bigint_mul(B(c), B(a), B(b))
        out.append([3000, 3000, to_int(c) == big * big, True, tail_zero(c), True])
        print(json.dumps({"cases": out, "dispatch": L.ntt_get_gpu_dispatch_count()}))
        L.ntt_mul_teardown_impl()
    """)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for case in res["cases"]:
        assert all(case[2:]), case
    assert res["dispatch"] == len(res["cases"])


def test_limb112_alias_square_managed_and_zero():
    r = run("""
        L.ntt_mul_init_impl(16)
        rng = random.Random(6)
        x, y = rnd(rng, 3000), rnd(rng, 2000)
        a, b = from_int(x, 6000), from_int(y)
        L.ntt_bigint_mul(B(a), B(a), B(b))               # c aliases a
        r1 = to_int(a) == x * y
        c = alloc(4)
        L.ntt_bigint_mul(B(c), B(b), B(b))               # a == b: squaring path
        r2 = to_int(c) == y * y
        L.ntt_bigint_sqr(B(c), B(b))
        r3 = to_int(c) == y * y
        m = L.bigint_alloc_managed(2500)                 # managed operand read where it is
        set_int(m, y)
        mo = L.bigint_alloc_managed(5000)                # managed output with room
        L.ntt_bigint_mul(B(mo), B(m), B(b))
        r4 = to_int(mo) == y * y and m.managed == 1
        zero = alloc(2)
        L.ntt_bigint_mul(B(c), B(zero), B(b))
        r5 = c.n_limbs == 0 and tail_zero(c)
        print(json.dumps([r1, r2, r3, r4, r5]))
        L.ntt_mul_teardown_impl()
    """)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1]) == [True] * 5


def test_limb112_wrap_guard_and_init_range():
    # test_wrap_guard.c's shape at 112-bit limbs: log_n = 12, 3000 + 3000 - 1
    # > 4096 must exit(1) before any kernel runs; 1000 + 1000 - 1 fits
    body = """
        L.ntt_mul_init_impl(12)
        a, b = from_int((1 << (112 * %d)) - 7), from_int((1 << (112 * %d)) - 9)
        c = alloc(8)
        L.ntt_bigint_mul(B(c), B(a), B(b))
        L.ntt_mul_teardown_impl()
        os._exit(0)
    """
    neg = run(body % (3000, 3000))
    assert neg.returncode == 1 and "exceed" in neg.stderr, (neg.returncode, neg.stderr)
    pos = run(body % (1000, 1000))
    assert pos.returncode == 0, pos.stderr
    r = run("L.ntt_mul_init_impl(29)\n")
    assert r.returncode == 1 and "out of safe range" in r.stderr
    r = run("a = from_int(5); c = alloc(4)\nL.ntt_bigint_mul(B(c), B(a), B(a))\n")
    assert r.returncode == 1 and "ntt_mul_init" in r.stderr


def test_limb112_managed_output_too_small_aborts_and_checked_codes():
    r = run("""
        L.ntt_mul_init_impl(12)
        a = from_int((1 << 1120) - 1)
        c = L.bigint_alloc_managed(2)
        L.ntt_bigint_mul(B(c), B(a), B(a))
    """)
    assert r.returncode != 0 and "pre-allocate larger" in r.stderr
    r = run("""
        L.ntt_mul_init_impl(10)
        a = from_int((1 << (112 * 1100)) - 3)
        c = alloc(4)
        print(json.dumps([L.ntt_bigint_mul_checked(B(c), B(a), B(a))]))
    """)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1]) == [2]   # GBNTT_ERR_SIZE
