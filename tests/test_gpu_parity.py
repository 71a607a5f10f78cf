"""GPU parity tests: every product computed by the CUDA engine is compared
bit-for-bit with the oracle (CPU CRT-NTT restatement), GMP mpz_mul and
Python integers, through the C ABI. Structure follows the reference's GPU
suites: test_polymul_sweep.hip (differential sweep across transform-size
boundaries, commutativity), test_gmp_oracle.c (full multiply vs mpz_mul),
test_ntt_kernel.hip (transform known answers)."""
import hashlib

import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart, synth

pytestmark = pytest.mark.gpu

SWEEP = [50, 65, 66, 80, 100, 127, 128, 129, 200, 256, 257, 400, 512, 513, 700, 1000, 1024, 1025, 1500, 2000,
         2048, 2049]   # ntt/app/compute_e/test_polymul_sweep.hip:114-115


def _rand(rng, n):
    return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)


def _full(c, n):
    out = np.zeros(n, dtype=np.uint32)
    out[:len(c)] = c
    return out


def _check(engine, a, b):
    got = engine.mul(a, b)
    want = _full(oracle.mul(a, b), len(a) + len(b))
    assert np.array_equal(got, want), (len(a), len(b), int(np.flatnonzero(got != want)[0]))
    return got


def test_small_and_tiny(engine):
    rng = np.random.default_rng(1)
    for na, nb in [(1, 1), (1, 2), (2, 1), (3, 5), (16, 17), (31, 1), (32, 1), (33, 33), (17, 16), (1, 64)]:
        _check(engine, _rand(rng, na), _rand(rng, nb))
    assert engine.device_errors() == 0


def test_sweep_vs_schoolbook(engine):
    rng = np.random.default_rng(2)
    for i, na in enumerate(SWEEP):
        for j, nb in enumerate(SWEEP):
            if (i + j) & 1:
                continue
            a, b = _rand(rng, na), _rand(rng, nb)
            got = engine.mul(a, b)
            assert np.array_equal(got, _full(oracle.schoolbook(a, b), na + nb)), (na, nb)
    assert engine.device_errors() == 0


@pytest.mark.parametrize("log_n", list(range(5, 25)))
def test_transform_length_boundaries(engine, log_n):
    # products whose coefficient count sits exactly on and just past 2^log_n,
    # covering every pass plan (1, 2 and 3 passes)
    rng = np.random.default_rng(100 + log_n)
    N = 1 << log_n
    for need in (N, N - 1, N + 1 if log_n < 24 else N):
        na = max(1, need // 2 + 3)
        nb = max(1, need + 1 - na)
        a, b = _rand(rng, na), _rand(rng, nb)
        got = engine.mul(a, b)
        if need <= 1 << 16:
            want = _full(oracle.mul(a, b), na + nb)
        else:
            want = _full(oracle.gmp_mul(a, b), na + nb)
        assert np.array_equal(got, want), (log_n, na, nb)
    assert engine.device_errors() == 0


def test_all_max_limbs(engine):
    # 0xFFFFFFFF everywhere: largest coefficients (near 2^93 scale) and
    # carries that ripple across tile boundaries of the carry scan
    for n in (1, 2, 1000, 2048, 2049, 4096, 100000, 1 << 20):
        a = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
        v = (1 << (32 * n)) - 1
        got = engine.mul(a, a)
        assert oracle.to_int(got) == v * v, n
    assert engine.device_errors() == 0


def test_long_carry_chains(engine):
    # a*b whose product is 2^k - 1 style patterns: (2^(32n) - 1) * 1 and
    # (2^(32n)-1) * (2^(32n)+1) = 2^(64n) - 1 with all-ones limbs
    for n in (100, 3000, 70000):
        ones = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
        one = np.array([1], dtype=np.uint32)
        assert np.array_equal(engine.mul(ones, one)[:n], ones)
        b = np.zeros(n + 1, dtype=np.uint32)
        b[0] = 1
        b[n] = 1
        got = engine.mul(ones, b)
        v = ((1 << (32 * n)) - 1) * ((1 << (32 * n)) + 1)
        assert oracle.to_int(got) == v
    assert engine.device_errors() == 0


def test_zero_and_untrimmed_operands(engine):
    rng = np.random.default_rng(4)
    a = _rand(rng, 500)
    z = np.zeros(300, dtype=np.uint32)
    assert not engine.mul(a, z).any()
    a2 = np.concatenate([a, np.zeros(77, dtype=np.uint32)])   # leading zero limbs
    got = engine.mul(a2, a)
    assert oracle.to_int(got) == oracle.to_int(a) ** 2
    assert len(engine.mul(np.zeros(0, dtype=np.uint32), a)) == 500


def test_square_and_commutativity(engine):
    rng = np.random.default_rng(5)
    for n in (1, 33, 1000, 4097, 1 << 17):
        a = _rand(rng, n)
        b = _rand(rng, n + 3)
        sq = engine.sqr(a)
        assert np.array_equal(sq, _full(oracle.square(a), 2 * n)), n
        assert np.array_equal(engine.mul(a, b), engine.mul(b, a)), n
    assert engine.device_errors() == 0


def test_unbalanced(engine):
    rng = np.random.default_rng(6)
    for na, nb in [(1, 1 << 20), (7, 1 << 19), (1 << 18, 1000)]:
        a, b = _rand(rng, na), _rand(rng, nb)
        assert np.array_equal(engine.mul(a, b), _full(oracle.gmp_mul(a, b), na + nb))


def test_golden_products(engine, golden):
    for pr in golden["products"]:
        a = synth.operand(pr["na"], pr["seed_a"])
        b = synth.operand(pr["nb"], pr["seed_b"])
        got = engine.mul(a, b)
        assert hashlib.sha256(got.astype("<u4").tobytes()).hexdigest() == pr["sha256"], (pr["na"], pr["nb"])


def test_config1_product_vs_gmp(engine):
    # 2^20 x 2^20 limbs, transform length 2^21 (the CPU-runnable configuration)
    a = synth.operand(1 << 20, 1)
    b = synth.operand(1 << 20, 2)
    got = engine.mul(a, b)
    assert np.array_equal(got, _full(oracle.gmp_mul(a, b), 1 << 21))
    assert np.array_equal(got, _full(oracle.mul(a, b), 1 << 21))


def test_2pow23_vs_gmp(engine):
    a = synth.operand(1 << 23, 3)
    b = synth.operand(1 << 23, 4)
    got = engine.mul(a, b)
    assert np.array_equal(got, _full(oracle.gmp_mul(a, b), 1 << 24))
    assert engine.device_errors() == 0


def test_device_pointer_api(engine):
    rng = np.random.default_rng(8)
    na, nb = 5000, 3001
    a, b = _rand(rng, na), _rand(rng, nb)
    da, db = cudart.DeviceBuffer(4 * na), cudart.DeviceBuffer(4 * nb)
    dc = cudart.DeviceBuffer(4 * max(na + nb, 2 * na))
    da.upload(a)
    db.upload(b)
    engine.mul_device(dc.ptr, da.ptr, na, db.ptr, nb, None)
    cudart.stream_sync(engine.lib().gbntt_stream())
    got = dc.download(np.uint32, na + nb)
    assert np.array_equal(got, _full(oracle.mul(a, b), na + nb))
    # square through the device API
    engine.lib().gbntt_sqr_u32(dc.ptr, da.ptr, na, None)
    cudart.stream_sync(engine.lib().gbntt_stream())
    assert np.array_equal(dc.download(np.uint32, 2 * na), _full(oracle.square(a), 2 * na))
    for buf in (da, db, dc):
        buf.free()


def _spectrum_positions(log_n):
    """Position of frequency k in the engine's forward output: the passes
    (outermost first) emit digit k_i of k = k_0 + L_0 k_1 + L_0 L_1 k_2 at
    stride N / (L_0 ... L_i)."""
    from cryptography_gb300 import engine as E
    passes = E.plan(log_n)
    k = np.arange(1 << log_n, dtype=np.int64)
    pos = np.zeros_like(k)
    rem = k.copy()
    stride = 1 << log_n
    for li in passes:
        stride >>= li
        pos += (rem & ((1 << li) - 1)) * stride
        rem >>= li
    return pos


@pytest.mark.parametrize("log_n", [5, 8, 10, 11, 14, 20, 21])
def test_forward_spectra_match_oracle(engine, log_n):
    # the engine's forward transform equals the oracle's natural-order DFT
    # (g^((p-1)/N) roots), up to the documented digit-reversed layout
    rng = np.random.default_rng(log_n)
    N = 1 << log_n
    n = N // 2 + 1
    x = _rand(rng, n)
    din = cudart.DeviceBuffer(4 * n)
    dout = cudart.DeviceBuffer(8 * 3 * N)
    din.upload(x)
    assert engine.lib().gbntt_debug_forward(dout.ptr, din.ptr, n, log_n, None) == 0
    cudart.stream_sync(engine.lib().gbntt_stream())
    got = dout.download(np.uint64, 3 * N).reshape(3, N)
    pos = _spectrum_positions(log_n)
    xin = np.zeros(N, dtype=np.uint64)
    xin[:n] = x
    for pi in range(3):
        want = oracle.ntt(pi, xin)
        assert np.array_equal(got[pi][pos], want), pi
    # KA1: delta_0 -> all ones; KA4: delta_1 -> w^k
    d = np.zeros(2, dtype=np.uint32)
    d[0] = 1
    din.upload(d)
    assert engine.lib().gbntt_debug_forward(dout.ptr, din.ptr, 1, log_n, None) == 0
    cudart.stream_sync(engine.lib().gbntt_stream())
    assert np.all(dout.download(np.uint64, 3 * N) == 1)
    d[0], d[1] = 0, 1
    din.upload(d)
    assert engine.lib().gbntt_debug_forward(dout.ptr, din.ptr, 2, log_n, None) == 0
    cudart.stream_sync(engine.lib().gbntt_stream())
    got = dout.download(np.uint64, 3 * N).reshape(3, N)
    for pi, p in enumerate(oracle.PRIMES):
        w = oracle.root(pi, log_n)
        kk = np.arange(N)
        sample = kk[:: max(1, N // 512)]
        assert all(int(got[pi][pos[k]]) == pow(w, int(k), p) for k in sample)
    din.free()
    dout.free()


def test_size_guard_native(engine):
    big = engine.lib().gbntt_max_log()
    with pytest.raises(engine.EngineError) as ei:
        engine.mul(np.ones((1 << big) // 2 + 2, dtype=np.uint32), np.ones((1 << big) // 2 + 2, dtype=np.uint32))
    assert ei.value.code == engine.GBNTT_ERR_SIZE


@pytest.mark.parametrize("prime", [0, 1, 2])
def test_device_modops(engine, prime):
    # the device modular arithmetic (PTX carry-chain forms and the plain C++
    # forms) against Python integers on random and corner operands, as the
    # reference's lib/test_modops.hip pins add/sub/mul for every prime
    p = oracle.PRIMES[prime]
    rng = np.random.default_rng(40 + prime)
    corners = [0, 1, 2, p - 1, p - 2, (1 << 32) - 1, 1 << 32, p >> 1, 1 << 63, p - (1 << 32)]
    n = 1 << 16
    a = np.array([int(x) % p for x in rng.integers(0, 1 << 64, n, dtype=np.uint64)], dtype=np.uint64)
    b = np.array([int(x) % p for x in rng.integers(0, 1 << 64, n, dtype=np.uint64)], dtype=np.uint64)
    k = len(corners)
    a[:k * k] = np.repeat(np.array(corners, dtype=np.uint64), k)
    b[:k * k] = np.tile(np.array(corners, dtype=np.uint64), k)
    wide = a.copy()
    wide[k * k:k * k + 100] = rng.integers(0, 1 << 64, 100, dtype=np.uint64) | np.uint64(1 << 63)
    wide[-4:] = [(1 << 64) - 1, (1 << 64) - 2, p, p + 1]
    da, db, dw, dout = (cudart.DeviceBuffer(8 * n) for _ in range(4))
    da.upload(a)
    db.upload(b)
    dw.upload(wide)
    rinv = pow(1 << 64, -1, p)
    want = {0: [(int(x) + int(y)) % p for x, y in zip(a, b)],
            1: [(int(x) - int(y)) % p for x, y in zip(a, b)],
            2: [int(x) * int(y) * rinv % p for x, y in zip(wide, b)]}
    for op in range(6):
        src = dw if op % 3 == 2 else da
        assert engine.lib().gbntt_debug_modops(prime, op, src.ptr, db.ptr, dout.ptr, n, None) == 0
        cudart.stream_sync(engine.lib().gbntt_stream())
        got = [int(v) for v in dout.download(np.uint64, n)]
        assert got == want[op % 3], (prime, op)
    for buf in (da, db, dw, dout):
        buf.free()


def test_device_pow2_q0(engine):
    # x * 2^e mod q0 (every e < 96) as the register DFTs multiply by powers
    # of two: the per-range forms against Python integers, corners included
    p = oracle.PRIMES[0]
    rng = np.random.default_rng(45)
    corners = [0, 1, 2, p - 1, p - 2, (1 << 32) - 1, 1 << 32, (1 << 63) - 1, 1 << 63, p - (1 << 32),
               (1 << 64) - (1 << 33), 0xFFFFFFFE00000001, 0x00000000FFFFFFFF, 0x80000000FFFFFFFF]
    per_e = 700
    xs = [c for c in corners] + [int(v) % p for v in rng.integers(0, 1 << 64, per_e - len(corners), dtype=np.uint64)]
    a = np.array(xs * 96, dtype=np.uint64)
    e = np.repeat(np.arange(96, dtype=np.uint64), per_e)
    n = len(a)
    da, de, dout = (cudart.DeviceBuffer(8 * n) for _ in range(3))
    da.upload(a)
    de.upload(e)
    assert engine.lib().gbntt_debug_modops(0, 6, da.ptr, de.ptr, dout.ptr, n, None) == 0
    cudart.stream_sync(engine.lib().gbntt_stream())
    got = [int(v) for v in dout.download(np.uint64, n)]
    want = [int(x) * pow(2, int(k), p) % p for x, k in zip(a, e)]
    bad = [i for i in range(n) if got[i] != want[i]]
    assert not bad, [(hex(int(a[i])), int(e[i]), hex(got[i]), hex(want[i])) for i in bad[:5]]
    for buf in (da, de, dout):
        buf.free()


def test_device_modops_lazy_q0(engine):
    # q0 in lazy normal form: operands are any 64-bit words (standing for
    # their value mod q0), results lie in [0, 2^64) and must agree mod q0
    p = oracle.PRIMES[0]
    rng = np.random.default_rng(44)
    corners = [0, 1, 2, p - 1, p, p + 1, (1 << 64) - 1, (1 << 64) - 2, (1 << 32) - 1, 1 << 32, 1 << 63,
               (1 << 64) - (1 << 32)]
    n = 1 << 16
    a = rng.integers(0, 1 << 64, n, dtype=np.uint64)
    b = rng.integers(0, 1 << 64, n, dtype=np.uint64)
    k = len(corners)
    a[:k * k] = np.repeat(np.array(corners, dtype=np.uint64), k)
    b[:k * k] = np.tile(np.array(corners, dtype=np.uint64), k)
    da, db, dout = (cudart.DeviceBuffer(8 * n) for _ in range(3))
    da.upload(a)
    db.upload(b)
    A = [int(x) for x in a]
    B = [int(y) for y in b]
    want = {0: [(x + y) % p for x, y in zip(A, B)], 1: [(x - y) % p for x, y in zip(A, B)],
            2: [x * y % p for x, y in zip(A, B)]}
    for op in range(6):
        assert engine.lib().gbntt_debug_modops(4, op, da.ptr, db.ptr, dout.ptr, n, None) == 0
        cudart.stream_sync(engine.lib().gbntt_stream())
        got = [int(v) for v in dout.download(np.uint64, n)]
        assert [v % p for v in got] == want[op % 3], op
        if op >= 3:
            assert got == want[op % 3], op   # the plain forms return canonical values
    for buf in (da, db, dout):
        buf.free()


def test_device_modops_p3(engine):
    # the 32-bit prime p3 = 3 * 2^30 + 1 (signed Montgomery, R = 2^32): PTX
    # and plain forms against Python integers, corners included
    p = 3 * (1 << 30) + 1
    rng = np.random.default_rng(43)
    corners = [0, 1, 2, p - 1, p - 2, (1 << 31) - 1, 1 << 31, p >> 1, (1 << 30), p - (1 << 30)]
    n = 1 << 16
    a = rng.integers(0, p, n, dtype=np.uint64)
    b = rng.integers(0, p, n, dtype=np.uint64)
    k = len(corners)
    a[:k * k] = np.repeat(np.array(corners, dtype=np.uint64), k)
    b[:k * k] = np.tile(np.array(corners, dtype=np.uint64), k)
    wide = a.copy()
    wide[k * k:k * k + 100] = rng.integers(p, 1 << 32, 100, dtype=np.uint64)
    wide[-3:] = [(1 << 32) - 1, p, p + 1]
    da, db, dw, dout = (cudart.DeviceBuffer(8 * n) for _ in range(4))
    da.upload(a)
    db.upload(b)
    dw.upload(wide)
    rinv = pow(1 << 32, -1, p)
    want = {0: [(int(x) + int(y)) % p for x, y in zip(a, b)],
            1: [(int(x) - int(y)) % p for x, y in zip(a, b)],
            2: [int(x) * int(y) * rinv % p for x, y in zip(wide, b)]}
    for op in range(6):
        src = dw if op % 3 == 2 else da
        assert engine.lib().gbntt_debug_modops(3, op, src.ptr, db.ptr, dout.ptr, n, None) == 0
        cudart.stream_sync(engine.lib().gbntt_stream())
        got = [int(v) for v in dout.download(np.uint64, n)]
        assert got == want[op % 3], op
    for buf in (da, db, dw, dout):
        buf.free()
