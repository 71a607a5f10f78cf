"""GPU tests of the reference-compatible entry points (ntt_mul_init_impl /
ntt_bigint_mul / ntt_mul_teardown_impl / ...) on the reference BigInt
layout. Each case runs in a child process, as the reference's death test
ntt/app/compute_e/test_wrap_guard.c forks one child per case: the engine is
process-global and the guard paths exit the process."""
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
    import cryptography_gb300 as g
    L = g.lib()
    B = ctypes.byref
    def rnd(rng, n):
        v = rng.getrandbits(64 * n) | (1 << (64 * n - 1)) if n else 0
        return v
""" % ROOT)


def run(body, env=None, timeout=300):
    e = dict(os.environ)
    e.pop("NTT_MAX_LOGN", None)
    if env:
        e.update(env)
    r = subprocess.run([sys.executable, "-c", PRELUDE + textwrap.dedent(body)], capture_output=True, text=True,
                       timeout=timeout, env=e)
    return r


def test_bigint_mul_matches_python_ints():
    r = run("""
        L.ntt_mul_init_impl(20)
        rng = random.Random(7)
        out = []
        for na, nb in [(1, 1), (2, 1), (33, 17), (1000, 999), (4096, 4096), (70000, 3), (1 << 18, (1 << 18) - 5)]:
            x, y = rnd(rng, na), rnd(rng, nb)
            a, b = g.bigint_from_int(x), g.bigint_from_int(y)
            c = g.bigint_alloc(1)                     # too small: the engine grows it
            L.ntt_bigint_mul(B(c), B(a), B(b))
            ok = g.bigint_to_int(c) == x * y
            tail = ctypes.string_at(c.limbs, 8 * c.cap)[8 * c.n_limbs:]
            out.append([na, nb, ok, c.cap >= na + nb + 4, set(tail) <= {0},
                        c.n_limbs == (x * y).bit_length() // 64 + (1 if (x * y).bit_length() % 64 else 0)])
            for v in (a, b, c):
                g.bigint_free(v)
        print(json.dumps({"cases": out, "dispatch": L.ntt_get_gpu_dispatch_count()}))
        L.ntt_mul_teardown_impl()
    """)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for case in res["cases"]:
        assert all(case[2:]), case
    assert res["dispatch"] == len(res["cases"])


def test_alias_square_and_managed():
    r = run("""
        L.ntt_mul_init_impl(16)
        rng = random.Random(11)
        x, y = rnd(rng, 3000), rnd(rng, 2000)
        a, b = g.bigint_from_int(x, 6000), g.bigint_from_int(y)
        L.ntt_bigint_mul(B(a), B(a), B(b))            # c aliases a
        r1 = g.bigint_to_int(a) == x * y
        s = g.bigint_from_int(y)
        c = g.bigint_alloc(8)
        L.ntt_bigint_mul(B(c), B(s), B(s))            # a == b: squaring path
        r2 = g.bigint_to_int(c) == y * y
        L.ntt_bigint_sqr(B(c), B(b))
        r3 = g.bigint_to_int(c) == y * y
        m = L.bigint_alloc_managed(4000)              # managed operand read in place
        g.bigint_set_int(m, y)
        mo = L.bigint_alloc_managed(8000)             # managed output with room
        L.ntt_bigint_mul(B(mo), B(m), B(s))
        r4 = g.bigint_to_int(mo) == y * y and m.managed == 1
        zero = g.bigint_alloc(2)
        L.ntt_bigint_mul(B(c), B(zero), B(s))
        r5 = c.n_limbs == 0
        print(json.dumps([r1, r2, r3, r4, r5]))
        g.bigint_free(m); g.bigint_free(mo)
        L.ntt_mul_teardown_impl()
    """)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1]) == [True] * 5


def test_managed_flag_on_host_heap_memory():
    # A reference build linked against the library dynamically keeps its own
    # weak bigint_alloc_managed (ntt/lib/arith/bigint.c:61-68): calloc'd host
    # memory with managed = 1. The engine must check what the memory is and
    # stage it, not hand it to the kernels as device-readable.
    r = run("""
        L.ntt_mul_init_impl(16)
        rng = random.Random(12)
        x, y = rnd(rng, 3000), rnd(rng, 2500)
        a = g.bigint_from_int(x, 3000)
        a.managed = 1                                 # calloc'd, flagged managed
        b = g.bigint_from_int(y, 2500)
        b.managed = 1
        c = g.bigint_alloc(6100)
        c.managed = 1                                 # managed output with room for both products
        L.ntt_bigint_mul(B(c), B(a), B(b))
        r1 = g.bigint_to_int(c) == x * y
        L.ntt_bigint_mul(B(c), B(a), B(a))            # square of a flagged operand
        r2 = g.bigint_to_int(c) == x * x
        print(json.dumps([r1, r2]))
        for v in (a, b, c):
            v.managed = 0
            g.bigint_free(v)
        L.ntt_mul_teardown_impl()
    """)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1]) == [True, True]


def test_wrap_guard_death():
    # ntt/app/compute_e/test_wrap_guard.c: log_n = 12 (N = 4096 64-bit
    # coefficients); 3000 + 3000 - 1 > N must exit(1) before any kernel runs,
    # 1000 + 1000 - 1 <= N must complete with exit 0.
    body = """
        L.ntt_mul_init_impl(12)
        a = g.bigint_alloc(%d + 4); b = g.bigint_alloc(%d + 4)
        for v, n in ((a, %d), (b, %d)):
            arr = (ctypes.c_uint64 * n).from_address(ctypes.addressof(v.limbs.contents))
            for i in range(n):
                arr[i] = i + 1
            v.n_limbs = n
        c = g.bigint_alloc((1 << 12) + 8)
        L.ntt_bigint_mul(B(c), B(a), B(b))
        L.ntt_mul_teardown_impl()
        os._exit(0)
    """
    neg = run(body % (3000, 3000, 3000, 3000))
    assert neg.returncode == 1, (neg.returncode, neg.stderr)
    assert "exceed" in neg.stderr
    pos = run(body % (1000, 1000, 1000, 1000))
    assert pos.returncode == 0, pos.stderr


def test_not_initialised_and_init_range():
    r = run("""
        a = g.bigint_from_int(5); c = g.bigint_alloc(4)
        L.ntt_bigint_mul(B(c), B(a), B(a))
    """)
    assert r.returncode == 1 and "ntt_mul_init" in r.stderr
    r = run("L.ntt_mul_init_impl(29)\n")      # above the default cap of 28
    assert r.returncode == 1 and "out of safe range" in r.stderr
    r = run("L.ntt_mul_init_impl(2)\n")
    assert r.returncode == 1
    r = run("L.ntt_mul_init_impl(12)\nL.ntt_mul_teardown_impl()\nL.ntt_mul_init_impl(14)\nprint('ok')\n",
            env={"NTT_MAX_LOGN": "14"})
    assert r.returncode == 0 and "ok" in r.stdout


def test_managed_output_too_small_aborts():
    r = run("""
        L.ntt_mul_init_impl(12)
        a = g.bigint_from_int((1 << 640) - 1)
        c = L.bigint_alloc_managed(2)
        L.ntt_bigint_mul(B(c), B(a), B(a))
    """)
    assert r.returncode != 0 and "pre-allocate larger" in r.stderr


def test_checked_variant_returns_codes():
    r = run("""
        L.ntt_mul_init_impl(10)
        a = g.bigint_alloc(1200)
        for i in range(1100):
            pass
        arr = (ctypes.c_uint64 * 1100).from_address(ctypes.addressof(a.limbs.contents))
        for i in range(1100):
            arr[i] = 3
        a.n_limbs = 1100
        c = g.bigint_alloc(4)
        rc = L.ntt_bigint_mul_checked(B(c), B(a), B(a))
        print(json.dumps([rc, L.gbntt_last_error().decode()[:20]]))
    """)
    assert r.returncode == 0, r.stderr
    rc, _ = json.loads(r.stdout.strip().splitlines()[-1])
    assert rc == 2   # GBNTT_ERR_SIZE


@pytest.mark.parametrize("zero_copy,stage", [("1", "1"), ("1", "0"), ("0", "1")])
def test_bigint_mul_pinned_host_buffers(zero_copy, stage):
    # page-locked BigInts: with zero copy the carry kernel writes the product
    # over NVLink-C2C and the operands are either read in place by the first
    # passes (stage 0) or staged in HBM (A by its first q0 pass, B by a copy
    # kernel on a second stream); without zero copy everything goes through
    # the staging buffer. All must give the exact product, squares included.
    r = run("""
        import numpy as np
        from cryptography_gb300 import cudart
        L.ntt_mul_init_impl(20)
        rng = random.Random(11)
        out = []
        u64p = ctypes.POINTER(ctypes.c_uint64)
        for na, nb in [(1, 1), (7, 5), (4096, 4093), ((1 << 18) + 3, (1 << 18) - 9)]:
            x, y = rnd(rng, na), rnd(rng, nb)
            pa, pb = cudart.PinnedBuffer(na, np.uint64), cudart.PinnedBuffer(nb, np.uint64)
            cap = max(na + nb, 2 * na) + 8   # room for the square too: no realloc of pinned memory
            pc = cudart.PinnedBuffer(cap, np.uint64)
            pa.array[:] = np.frombuffer(x.to_bytes(8 * na, "little"), dtype=np.uint64)
            pb.array[:] = np.frombuffer(y.to_bytes(8 * nb, "little"), dtype=np.uint64)
            pc.array[:] = 0xAAAAAAAAAAAAAAAA
            a = g.BigInt(ctypes.cast(pa.ptr, u64p), na, na, 0)
            b = g.BigInt(ctypes.cast(pb.ptr, u64p), nb, nb, 0)
            c = g.BigInt(ctypes.cast(pc.ptr, u64p), 0, cap, 0)
            L.ntt_bigint_mul(B(c), B(a), B(b))
            ok = int.from_bytes(pc.array[:c.n_limbs].tobytes(), "little") == x * y
            out.append([na, nb, ok, int(c.limbs[0] == pc.array[0]), bool((pc.array[c.n_limbs:] == 0).all())])
            pc.array[:] = 0
            L.ntt_bigint_mul(B(c), B(a), B(a))
            ok = int.from_bytes(pc.array[:c.n_limbs].tobytes(), "little") == x * x
            out.append([na, na, ok, int(c.limbs[0] == pc.array[0]), c.cap == cap])
            for p in (pa, pb, pc):
                p.free()
        print(json.dumps(out))
        L.ntt_mul_teardown_impl()
    """, env={"GBNTT_ZERO_COPY": zero_copy, "GBNTT_STAGE_INPUTS": stage})
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(ok and same and zeros for _, _, ok, same, zeros in res), res
