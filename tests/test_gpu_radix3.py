"""Transforms of length 3 2^k: a product whose coefficient count fits
3 2^k but not 2^(k+1) runs the radix-3 stage (gbntt_radix3.cu) around
three 2^k-point pass chains instead of one 2^(k+2)-point transform. Every
such product is compared bit-for-bit with the oracle (GMP above 2^16
coefficients), on both sides of the 3 2^k boundary, through the host and
device entry points, squares, all-ones operands (the largest coefficients)
and batches mixing radix-3 waves with paired, shared and power-of-two ones.
The launch log shows which path ran."""
import os

import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def r3engine(engine):
    """The engine with radix-3 transforms from 3 2^10 points for every
    product (GBNTT_RADIX3_MIN_LOG=10; by default only sizes where they are
    faster take them), restored to the default afterwards."""
    engine.teardown()
    os.environ["GBNTT_RADIX3_MIN_LOG"] = "10"
    try:
        engine.init(24)
        yield engine
    finally:
        os.environ.pop("GBNTT_RADIX3_MIN_LOG", None)
        engine.teardown()
        engine.init(24)


def _rand(rng, n):
    return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)


def _want(a, b):
    r = oracle.mul(a, b) if len(a) + len(b) <= (1 << 16) else oracle.gmp_mul(a, b)
    out = np.zeros(len(a) + len(b), dtype=np.uint32)
    out[:len(r)] = r
    return out


def _kinds(engine, fn):
    engine.launch_log(True)
    try:
        fn()
        return {r[0] for r in engine.launch_records(1 << 16)}
    finally:
        engine.launch_log(False)


def _upload(arrs):
    bufs = []
    for a in arrs:
        b = cudart.DeviceBuffer(max(4, 4 * len(a)))
        if len(a):
            b.upload(a)
        bufs.append(b)
    return bufs


def test_radix3_default_threshold(engine):
    # (first in the module: it needs the default engine, before r3engine)
    # default rule: a product alone takes the radix-3 transform from 3 2^20
    # points; a batch for c products of 3 2^k points when c 2^k >= 2^20
    rng = np.random.default_rng(37)
    small = (_rand(rng, 3000), _rand(rng, 3000))                  # 3 2^11 points
    kinds = _kinds(engine, lambda: engine.mul(*small))
    assert not kinds & {"radix3_fwd", "radix3_inv"}, kinds
    n = 3 << 19                                                   # 2 n - 1 <= 3 2^20
    big = (_rand(rng, n), _rand(rng, n - 5))
    kinds = _kinds(engine, lambda: engine.mul(*big))
    assert {"radix3_fwd", "radix3_inv"} <= kinds, kinds
    assert np.array_equal(engine.mul(*big), _want(*big))
    for count, expect in ((255, False), (256, True)):              # 6000 x 6000: 3 2^12 points
        A = [_rand(rng, 6000) for _ in range(count)]
        B = [_rand(rng, 6000) for _ in range(count)]
        da, db = _upload(A), _upload(B)
        dc = [cudart.DeviceBuffer(4 * 12000) for _ in A]
        kinds = _kinds(engine, lambda: (engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da],
                                                                [6000] * count, [x.ptr for x in db],
                                                                [6000] * count), cudart.synchronize()))
        assert bool(kinds & {"radix3_fwd"}) == expect, (count, kinds)
        for i in range(0, count, 51):
            assert np.array_equal(dc[i].download(np.uint32, 12000), _want(A[i], B[i])), (count, i)
        for x in da + db + dc:
            x.free()
    assert engine.device_errors() == 0


Q0 = (1 << 64) - (1 << 32) + 1
P3 = 3 * (1 << 30) + 1


def _cyclic(a, b, n):
    # exact coefficients of the linear convolution by Kronecker substitution
    # (96-bit slots), folded mod X^n - 1
    A = int.from_bytes(b"".join(int(x).to_bytes(12, "little") for x in a), "little")
    B = int.from_bytes(b"".join(int(x).to_bytes(12, "little") for x in b), "little")
    C = (A * B).to_bytes(12 * (len(a) + len(b)), "little")
    out = [0] * n
    for i in range(len(a) + len(b) - 1):
        out[i % n] += int.from_bytes(C[12 * i:12 * i + 12], "little")
    return out


@pytest.mark.parametrize("k", [10, 11, 13])
def test_radix3_stage_residues(r3engine, k):
    # the radix-3 stages alone give 3 a (mode 0: the 1/3 is applied by the
    # inverse sub-transforms' scale), and the whole
    # transform path gives the cyclic convolution mod q0 and p3 (mode 1),
    # for operands that fill all three thirds and for short ones
    rng = np.random.default_rng(900 + k)
    M3 = 3 << k
    for na, nb, mode in ((M3, 1, 0), (M3 // 2, M3 // 2, 1), (M3 // 2 + 1, M3 // 2, 1), (100, 77, 1)):
        a, b = _rand(rng, na), _rand(rng, nb)
        da, db = _upload([a, b])
        dq, dp = cudart.DeviceBuffer(8 * M3), cudart.DeviceBuffer(4 * M3)
        assert r3engine.lib().gbntt_debug_radix3(dq.ptr, dp.ptr, da.ptr, na, db.ptr, nb, k, mode) == 0
        q, p = dq.download(np.uint64, M3), dp.download(np.uint32, M3)
        want = [3 * int(x) for x in a] + [0] * (M3 - na) if mode == 0 else _cyclic(a, b, M3)
        assert [int(x) % Q0 for x in q] == [v % Q0 for v in want], (k, na, nb, mode)
        assert [int(x) % P3 for x in p] == [v % P3 for v in want], (k, na, nb, mode)
        for x in (da, db, dq, dp):
            x.free()


@pytest.mark.parametrize("k", list(range(10, 23)))
def test_radix3_lengths_match_oracle(r3engine, k):
    engine = r3engine
    rng = np.random.default_rng(300 + k)
    top = 3 << k
    for need in (top, top - 1, (1 << (k + 1)) + 1, top + 1):
        for na in (need // 2 + 1, max(1, need // 7)):
            nb = need + 1 - na
            a, b = _rand(rng, na), _rand(rng, nb)
            assert np.array_equal(engine.mul(a, b), _want(a, b)), (k, na, nb)
    assert engine.device_errors() == 0


def test_radix3_path_is_taken(r3engine):
    engine = r3engine
    rng = np.random.default_rng(7)
    a, b = _rand(rng, 3000), _rand(rng, 3000)      # 5999 <= 3 2^11
    kinds = _kinds(engine, lambda: engine.mul(a, b))
    assert {"radix3_fwd", "radix3_inv"} <= kinds, kinds
    c, d = _rand(rng, 3100), _rand(rng, 3100)      # 6199 > 3 2^11: 2^13 points
    kinds = _kinds(engine, lambda: engine.mul(c, d))
    assert not kinds & {"radix3_fwd", "radix3_inv"}, kinds
    a2, b2 = _rand(rng, 700), _rand(rng, 700)      # below 3 2^10 coefficients: power of two
    kinds = _kinds(engine, lambda: engine.mul(a2, b2))
    assert not kinds & {"radix3_fwd", "radix3_inv"}, kinds


def test_radix3_all_max_and_squares(r3engine):
    engine = r3engine
    for k in (10, 13, 17, 21):
        n = 3 << (k - 1)                            # 2 n - 1 = 3 2^k - 1 coefficients
        full = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
        c = engine.mul(full, full)                  # same array: the squaring path
        assert c[0] == 1 and not c[1:n].any() and c[n] == 0xFFFFFFFE and (c[n + 1:] == 0xFFFFFFFF).all(), k
        c2 = engine.mul(full, full.copy())
        assert np.array_equal(c, c2), k
    rng = np.random.default_rng(17)
    a = _rand(rng, 40000)
    assert np.array_equal(engine.sqr(a), _want(a, a))
    assert engine.device_errors() == 0


def test_radix3_device_pointers_and_aliasing(r3engine):
    engine = r3engine
    rng = np.random.default_rng(19)
    a, b = _rand(rng, 50000), _rand(rng, 45000)    # 94999 <= 3 2^15
    da, db = _upload([a, b])
    dc = cudart.DeviceBuffer(4 * (len(a) + len(b)))
    engine.mul_device(dc.ptr, da.ptr, len(a), db.ptr, len(b))
    cudart.synchronize()
    want = _want(a, b)
    assert np.array_equal(dc.download(np.uint32, len(a) + len(b)), want)
    big = cudart.DeviceBuffer(4 * (len(a) + len(b)))    # c aliases a
    big.upload(a)
    engine.mul_device(big.ptr, big.ptr, len(a), db.ptr, len(b))
    cudart.synchronize()
    assert np.array_equal(big.download(np.uint32, len(a) + len(b)), want)
    for x in (da, db, dc, big):
        x.free()
    assert engine.device_errors() == 0


def test_radix3_pinned_host_operands(r3engine):
    engine = r3engine
    # pinned operands and result: the zero-copy staging of A and B (copy
    # kernel over NVLink-C2C) in front of the radix-3 stage
    rng = np.random.default_rng(23)
    na, nb = 3 << 17, (3 << 17) - 1000          # both products <= 3 2^18 coefficients
    pa, pb = cudart.PinnedBuffer(na, np.uint32), cudart.PinnedBuffer(nb, np.uint32)
    pc = cudart.PinnedBuffer(2 * na, np.uint32)
    pa.array[:] = _rand(rng, na)
    pb.array[:] = _rand(rng, nb)
    from cryptography_gb300 import engine as eng
    import ctypes
    p = ctypes.POINTER(ctypes.c_uint32)
    for x, y, n_x, n_y in ((pa, pb, na, nb), (pa, pa, na, na)):
        call = lambda: eng._check(eng.lib().gbntt_mul_u32_host(ctypes.cast(pc.ptr, p), ctypes.cast(x.ptr, p), n_x,
                                                              ctypes.cast(y.ptr, p), n_y))
        kinds = _kinds(engine, call)
        assert {"radix3_fwd", "radix3_inv"} <= kinds, kinds
        assert np.array_equal(pc.array[:n_x + n_y], _want(x.array, y.array)), (n_x, n_y)
        call()                                  # again with the second stream (no launch log)
        assert np.array_equal(pc.array[:n_x + n_y], _want(x.array, y.array)), (n_x, n_y)
    for x in (pa, pb, pc):
        x.free()
    assert engine.device_errors() == 0


def test_radix3_batches(r3engine):
    engine = r3engine
    # a batch mixing radix-3 products with power-of-two ones, pairs sharing
    # a right operand (one transform per pair, per sub-transform for 3 2^k
    # points) and a run sharing one right operand, whose radix-3 and
    # power-of-two lengths become two waves each transforming it once; two
    # rounds so the second replays the wave graphs
    rng = np.random.default_rng(29)
    shared = _rand(rng, 2000)
    pair_b = _rand(rng, 5000)
    pair_c = _rand(rng, 3000)
    for rnd in range(2):
        A, B = [], []
        for n in rng.integers(1100, 30000, 24):
            A.append(_rand(rng, int(n)))
            B.append(_rand(rng, int(rng.integers(1100, 30000))))
        for n in (4000, 4000, 4300, 4100, 4300, 3900):   # 5999 / 6099 <= 3 2^11; 6299 > 3 2^11
            A.append(_rand(rng, n))
            B.append(shared)
        A += [_rand(rng, 5000), _rand(rng, 4500)]        # a pair at 3 2^12 points
        B += [pair_b, pair_b]
        A += [_rand(rng, 3000), _rand(rng, 3200)]        # a pair split by length: 5999 and 6199
        B += [pair_c, pair_c]
        da, db = _upload(A), _upload(B)
        dc = [cudart.DeviceBuffer(4 * (len(a) + len(b))) for a, b in zip(A, B)]
        call = lambda: engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                                               [x.ptr for x in db], [len(b) for b in B])
        if rnd == 0:
            kinds = _kinds(engine, lambda: (call(), cudart.synchronize()))
            assert {"radix3_fwd", "radix3_inv"} <= kinds, kinds
        else:
            call()
        cudart.synchronize()
        for i, (a, b, c) in enumerate(zip(A, B, dc)):
            got = c.download(np.uint32, len(a) + len(b))
            assert np.array_equal(got, _want(a, b)), (rnd, i, len(a), len(b))
        for x in da + db + dc:
            x.free()
    assert engine.device_errors() == 0


def test_radix3_batch_one_size(r3engine):
    engine = r3engine
    # 200 products of 6000 x 6000 limbs (11999 <= 3 2^12 coefficients): one
    # radix-3 wave of 200 products, each equal to the single product
    rng = np.random.default_rng(31)
    A = [_rand(rng, 6000) for _ in range(200)]
    B = [_rand(rng, 6000) for _ in range(200)]
    da, db = _upload(A), _upload(B)
    dc = [cudart.DeviceBuffer(4 * 12000) for _ in A]
    engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [6000] * 200, [x.ptr for x in db],
                            [6000] * 200)
    cudart.synchronize()
    for i in range(0, 200, 17):
        assert np.array_equal(dc[i].download(np.uint32, 12000), _want(A[i], B[i])), i
    for i in range(200):
        assert np.array_equal(dc[i].download(np.uint32, 12000), engine.mul(A[i], B[i])), i
    for x in da + db + dc:
        x.free()
    assert engine.device_errors() == 0



def test_radix3_shared_and_paired_waves_alone(r3engine):
    # batches made only of products sharing one right operand (radix-3 and
    # power-of-two lengths: two shared waves) and only of pairs (radix-3
    # pairs: the right operands' sub-transforms shared per pair)
    engine = r3engine
    rng = np.random.default_rng(41)
    b = _rand(rng, 2000)
    A = [_rand(rng, n) for n in (4000, 4100, 4300, 3900, 4000, 4300, 2500)]
    B = [b] * len(A)
    bs = [_rand(rng, 7000 + 50 * i) for i in range(4)]
    A2, B2 = [], []
    for i, bb in enumerate(bs):                        # pairs: n + 7000.. - 1 <= 3 2^12
        A2 += [_rand(rng, 5000 - 100 * i), _rand(rng, 4800 - 100 * i)]
        B2 += [bb, bb]
    for AA, BB in ((A, B), (A2, B2)):
        da, db = _upload(AA), _upload(BB)
        dc = [cudart.DeviceBuffer(4 * (len(x) + len(y))) for x, y in zip(AA, BB)]
        call = lambda: (engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(x) for x in AA],
                                                [x.ptr for x in db], [len(y) for y in BB]), cudart.synchronize())
        kinds = _kinds(engine, call)
        assert {"radix3_fwd", "radix3_inv"} <= kinds, kinds
        call()                                         # again without the launch log (second stream)
        for i, (x, y, c) in enumerate(zip(AA, BB, dc)):
            assert np.array_equal(c.download(np.uint32, len(x) + len(y)), _want(x, y)), (i, len(x), len(y))
        for buf in da + db + dc:
            buf.free()
    assert engine.device_errors() == 0
