"""Batched products (gbntt_batch_mul_u32): every product of a mixed batch
must be bit-identical to the same product computed alone (gbntt_mul_u32) and
to the oracle; buckets larger than one wave exercise the wave loop and the
table slots; empty operands give zero products."""
import numpy as np
import pytest

import oracle
from cryptography_gb300 import cudart

pytestmark = pytest.mark.gpu


def _upload(arrs):
    bufs = []
    for a in arrs:
        b = cudart.DeviceBuffer(max(4, 4 * len(a)))
        if len(a):
            b.upload(a)
        bufs.append(b)
    return bufs


def _run_batch(engine, A, B):
    da, db = _upload(A), _upload(B)
    dc = [cudart.DeviceBuffer(max(4, 4 * (len(a) + len(b)))) for a, b in zip(A, B)]
    engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                            [x.ptr for x in db], [len(b) for b in B])
    cudart.synchronize()
    out = [c.download(np.uint32, len(a) + len(b)) for c, a, b in zip(dc, A, B)]
    for buf in da + db + dc:
        buf.free()
    return out


def test_batch_mixed_sizes_match_single(engine):
    rng = np.random.default_rng(123)
    sizes = [int(x) for x in np.exp(rng.uniform(np.log(1), np.log(20000), 300))] + [1 << 16, 70000, 1 << 17]
    A, B = [], []
    for s in sizes:
        na = max(1, s)
        nb = max(1, int(s * rng.uniform(0.3, 1.5)))
        A.append(rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32))
        B.append(rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32))
    got = _run_batch(engine, A, B)
    for i, (a, b, c) in enumerate(zip(A, B, got)):
        assert np.array_equal(c, engine.mul(a, b)), i
    for i in range(0, len(A), 37):
        want = np.zeros(len(A[i]) + len(B[i]), dtype=np.uint32)
        r = oracle.mul(A[i], B[i])
        want[:len(r)] = r
        assert np.array_equal(got[i], want), i
    assert engine.device_errors() == 0


def test_batch_multi_wave_bucket(engine):
    # the engine fixture holds 2^24 coefficients: products of 2^20 coefficients
    # run 16 per wave, so 40 of them take 3 waves
    rng = np.random.default_rng(9)
    A = [rng.integers(0, 1 << 32, (1 << 19) - 7 - i, dtype=np.uint64).astype(np.uint32) for i in range(40)]
    B = [rng.integers(0, 1 << 32, (1 << 19) + 3, dtype=np.uint64).astype(np.uint32) for _ in range(40)]
    got = _run_batch(engine, A, B)
    for i in (0, 1, 15, 16, 17, 31, 32, 39):
        assert np.array_equal(got[i], engine.mul(A[i], B[i])), i
    assert engine.device_errors() == 0


def test_batch_empty_and_all_max(engine):
    A = [np.zeros(0, dtype=np.uint32), np.full(3000, 0xFFFFFFFF, dtype=np.uint32), np.array([5], dtype=np.uint32)]
    B = [np.arange(1, 11, dtype=np.uint32), np.full(2000, 0xFFFFFFFF, dtype=np.uint32), np.zeros(0, dtype=np.uint32)]
    got = _run_batch(engine, A, B)
    assert not got[0].any() and not got[2].any()
    v1, v2 = (1 << (32 * 3000)) - 1, (1 << (32 * 2000)) - 1
    assert oracle.to_int(got[1]) == v1 * v2


def test_device_operand_generator_matches_host(engine):
    from cryptography_gb300 import synth
    for n, seed in ((1, 3), (1000, 7), (1 << 20, 11)):
        d = cudart.DeviceBuffer(4 * n)
        assert engine.lib().gbntt_fill_operand(d.ptr, n, seed, None) == 0
        cudart.synchronize()
        assert np.array_equal(d.download(np.uint32, n), synth.operand(n, seed))
        d.free()


def test_batch_many_tiny_products_on_a_small_engine():
    # a wave of W tiny products needs W carry tiles although W 2^L fits a
    # small workspace: the status area must hold them (2^16 engine, W = 2048)
    import json
    import os
    import subprocess
    import sys
    import textwrap
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    body = textwrap.dedent("""
        import json, sys
        sys.path.insert(0, %r)
        import numpy as np
        import cryptography_gb300 as g
        from cryptography_gb300 import cudart
        g.init(16)
        rng = np.random.default_rng(77)
        n = 5000
        A = [rng.integers(0, 1 << 32, int(rng.integers(1, 16)), dtype=np.uint64).astype(np.uint32) for _ in range(n)]
        B = [rng.integers(0, 1 << 32, int(rng.integers(1, 16)), dtype=np.uint64).astype(np.uint32) for _ in range(n)]
        bufs = []
        def up(a):
            b = cudart.DeviceBuffer(max(4, 4 * len(a))); b.upload(a); bufs.append(b); return b
        da = [up(a) for a in A]; db = [up(b) for b in B]
        dc = [cudart.DeviceBuffer(4 * (len(a) + len(b))) for a, b in zip(A, B)]
        g.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                           [x.ptr for x in db], [len(b) for b in B])
        cudart.synchronize()
        ok = all(np.array_equal(c.download(np.uint32, len(a) + len(b)), g.mul(a, b)) for c, a, b in zip(dc, A, B))
        print(json.dumps([ok, g.device_errors()]))
    """ % root)
    r = subprocess.run([sys.executable, "-c", body], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert json.loads(r.stdout.strip().splitlines()[-1]) == [True, 0]


def test_batch_shared_right_operand(engine):
    # every product of the batch multiplies by the same device operand (the
    # e pipeline's divisions by a shared reciprocal or divisor): its
    # transform is computed once per wave; results must equal single
    # products. Two rounds so the second replays the wave graphs.
    rng = np.random.default_rng(31)
    for nb in (1, 700, 5000):
        b = rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32)
        db = _upload([b])[0]
        for _ in range(2):
            A = [rng.integers(0, 1 << 32, int(n), dtype=np.uint64).astype(np.uint32)
                 for n in rng.integers(1, 6000, 40)]
            da = _upload(A)
            dc = [cudart.DeviceBuffer(max(4, 4 * (len(a) + nb))) for a in A]
            engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                                    [db.ptr] * len(A), [nb] * len(A))
            cudart.synchronize()
            got = [c.download(np.uint32, len(a) + nb) for c, a in zip(dc, A)]
            for i, (a, c) in enumerate(zip(A, got)):
                assert np.array_equal(c, engine.mul(a, b)), (nb, i)
            for i in range(0, len(A), 13):
                want = np.zeros(len(A[i]) + nb, dtype=np.uint32)
                r = oracle.mul(A[i], b)
                want[:len(r)] = r
                assert np.array_equal(got[i], want), (nb, i)
            for x in da + dc:
                x.free()
        db.free()
    assert engine.device_errors() == 0


def test_batch_uneven_products_split(engine):
    # lopsided pairs (longer operand >= 8x the shorter, shorter >= 64 limbs)
    # run as chunk products of the shorter operand's size plus one addition;
    # both operand orders, the size thresholds, thousands of chunks, and a
    # mix with balanced products: every result must equal the single
    # product (which runs one full-length transform) and GMP
    rng = np.random.default_rng(808)
    shapes = [(100000, 64), (64, 100000), ((1 << 18) + 5, 3000), (5000, (1 << 17) - 3),
              (70000, 63), (4096, 512), (4095, 512), ((1 << 20) + 11, 100), (3000, 2900),
              (1 << 16, 1 << 16), (200, 1 << 15), (1 << 19, 1 << 12)]
    A, B = [], []
    for na, nb in shapes:
        A.append(rng.integers(0, 1 << 32, na, dtype=np.uint64).astype(np.uint32))
        B.append(rng.integers(0, 1 << 32, nb, dtype=np.uint64).astype(np.uint32))
    A.append(np.full(1 << 17, 0xFFFFFFFF, dtype=np.uint32))   # all-ones: longest carries
    B.append(np.full(700, 0xFFFFFFFF, dtype=np.uint32))
    for _ in range(2):   # the second round replays the wave graphs
        got = _run_batch(engine, A, B)
        for i, (a, b, c) in enumerate(zip(A, B, got)):
            want = np.zeros(len(a) + len(b), dtype=np.uint32)
            r = oracle.gmp_mul(a, b)
            want[:len(r)] = r
            assert np.array_equal(c, want), (i, len(a), len(b))
            if i % 3 == 0:
                assert np.array_equal(c, engine.mul(a, b)), i
    assert engine.device_errors() == 0


def _run_batch_shared(engine, A, B, bidx):
    # product i multiplies A[i] by B[bidx[i]] (one device buffer per B)
    da, db = _upload(A), _upload(B)
    nb = [len(B[j]) for j in bidx]
    dc = [cudart.DeviceBuffer(max(4, 4 * (len(a) + n))) for a, n in zip(A, nb)]
    engine.batch_mul_device([c.ptr for c in dc], [x.ptr for x in da], [len(a) for a in A],
                            [db[j].ptr for j in bidx], nb)
    cudart.synchronize()
    out = [c.download(np.uint32, len(a) + n) for c, a, n in zip(dc, A, nb)]
    for buf in da + db + dc:
        buf.free()
    return out


def test_batch_pairs_sharing_right_operand(engine):
    # Neighbours that multiply by the same right operand (a product tree's
    # B_L B_R and P_L B_R) run as pairs whose right operand is transformed
    # once: pairs of equal and of different left lengths, pairs whose two
    # products land on different transform lengths (not paired), lone
    # products between them, and a bucket of pairs longer than one wave
    # (waves must split between pairs).
    rng = np.random.default_rng(77)

    def rnd(n):
        return rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)

    A, B, bidx = [], [], []
    for k in range(60):
        nr = int(rng.integers(1, 30000))
        B.append(rnd(nr))
        na1 = int(rng.integers(1, 30000))
        na2 = na1 + int(rng.integers(-2, 3)) if k % 3 else int(rng.integers(1, 30000))
        A += [rnd(max(1, na1)), rnd(max(1, na2))]
        bidx += [len(B) - 1, len(B) - 1]
        if k % 7 == 0:   # a lone product between pairs
            A.append(rnd(int(rng.integers(1, 5000))))
            B.append(rnd(int(rng.integers(1, 5000))))
            bidx.append(len(B) - 1)
        if k % 11 == 0:  # a lone product by a copy of its own right operand
            A.append(B[-1].copy())
            bidx.append(len(B) - 1)
    # straddling a power of two: 4096 + 4097 - 1 = 2^13 coefficients, 4097 + 4097 - 1 above it
    B.append(rnd(4097))
    A += [rnd(4096), rnd(4097)]
    bidx += [len(B) - 1, len(B) - 1]
    # a bucket of 40 pairs of 2^20-coefficient products (16 per wave at 2^24)
    for k in range(40):
        B.append(rnd((1 << 19) + 3))
        A += [rnd((1 << 19) - 7 - k), rnd((1 << 19) - 9 - k)]
        bidx += [len(B) - 1, len(B) - 1]
    got = _run_batch_shared(engine, A, B, bidx)
    for i, (a, j, c) in enumerate(zip(A, bidx, got)):
        if len(a) > (1 << 18) and i % 5:
            continue
        assert np.array_equal(c, engine.mul(a, B[j])), i
    for i in range(0, len(A), 17):
        want = np.zeros(len(A[i]) + len(B[bidx[i]]), dtype=np.uint32)
        r = oracle.mul(A[i], B[bidx[i]])
        want[:len(r)] = r
        assert np.array_equal(got[i], want), i
    assert engine.device_errors() == 0
