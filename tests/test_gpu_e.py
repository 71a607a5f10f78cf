"""GPU parity of the e pipeline and the arith layer above the multiply,
through the C ABI: binary splitting, Newton reciprocal, division, powers of
ten and decimal conversion against Python integers and the e oracle, and
compute_e's digits against the reference's own output (sha256 in
tests/golden/e_digits.json)."""
import hashlib
import json
import os
import random
import subprocess
import sys
import textwrap

import pytest

from oracle import e_oracle as eo

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "e_digits.json")

if hasattr(sys, "set_int_max_str_digits"):
    sys.set_int_max_str_digits(0)


@pytest.fixture(scope="module")
def e_gold():
    with open(GOLD) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def arith(engine):
    from cryptography_gb300 import arith as a
    return a


def _rand(rng, nlimbs, top=None):
    v = rng.getrandbits(32 * nlimbs)
    if top is not None:
        v = (v & ((1 << (32 * (nlimbs - 1))) - 1)) | (top << (32 * (nlimbs - 1)))
    return v | (1 << (32 * nlimbs - 1)) if top is None else v


def test_binary_split_matches_oracle(arith, engine):
    cases = [(1, 1), (5, 3), (1, 2), (1, 3), (2, 3), (1, 63), (1, 64), (1, 65), (1, 129), (3, 1000),
             (1, 5000), (1000, 1001), (12345, 23456), (1, 20000), ((1 << 32) - 200, 1 << 32)]
    for a, b in cases:
        assert arith.binary_split(a, b) == eo.binary_split_seq(a, b), (a, b)
    assert engine.device_errors() == 0


@pytest.mark.parametrize("levels", ["0", "1", "3", "6", "8"])
def test_binary_split_block_levels(arith, engine, levels, monkeypatch):
    # GBNTT_BS_BLOCK_LEVELS levels of the tree are merged in shared memory
    # (groups of 64 terms, 2^levels per CTA, empty groups past the end);
    # ranges that end mid-group, mid-CTA, and terms near 2^32.
    monkeypatch.setenv("GBNTT_BS_BLOCK_LEVELS", levels)
    for a, b in [(1, 2), (1, 64), (1, 65), (1, 4097), (7, 70000), (1, 300001), (123456, 123456 + 8191),
                 ((1 << 32) - 5000, 1 << 32)]:
        assert arith.binary_split(a, b) == eo.binary_split(a, b), (levels, a, b)
    assert engine.device_errors() == 0


@pytest.mark.parametrize("wrap", ["0", "1"])
def test_newton_reciprocal(arith, wrap, monkeypatch):
    # wrap 1: the exactness check takes beta^(2k) - Y T from a cyclic product
    monkeypatch.setenv("GBNTT_E_WRAP", wrap)
    rng = random.Random(5)
    vals = [1, 2, 3, 5, 2 ** 31, 2 ** 32 - 1, 2 ** 32, 2 ** 32 + 1, 2 ** 64 - 1, 2 ** 64, 2 ** 95 + 12345,
            2 ** (32 * 7), 2 ** (32 * 7) - 1, 3 ** 500, 10 ** 1000, 2 ** 4095, 2 ** 4096 - 1]
    for nl in [1, 2, 3, 4, 5, 7, 8, 15, 16, 17, 33, 100, 257, 1000, 4097, 20000]:
        vals.append(_rand(rng, nl))
        vals.append(_rand(rng, nl, top=1))
        vals.append(_rand(rng, nl, top=0xFFFFFFFF))
    for q in vals:
        assert arith.newton_reciprocal(q) == eo.newton_reciprocal(q), q.bit_length()


@pytest.mark.parametrize("wrap", ["0", "1"])
def test_div_newton(arith, wrap, monkeypatch):
    # wrap 1: remainders from cyclic products mod beta^W - 1 where shorter
    monkeypatch.setenv("GBNTT_E_WRAP", wrap)
    rng = random.Random(6)
    cases = [(0, 7), (5, 7), (7, 7), (8, 7), (2 ** 64, 1), (10 ** 50, 2 ** 40), (2 ** 1000 - 1, 2 ** 500)]
    for nn, nd in [(1, 1), (2, 1), (3, 2), (10, 3), (100, 50), (100, 99), (101, 51), (1000, 10), (5000, 1000),
                   (20000, 10000), (20001, 10000), (30000, 7000), (4000, 3999), (60000, 20000)]:
        n = _rand(rng, nn)
        d = _rand(rng, nd, top=rng.choice([1, 0x80000000, 0xFFFFFFFF, rng.getrandbits(32) | 1]))
        cases.append((n, d))
        q = n // d
        cases.append((q * d, d))            # zero remainder
        cases.append((q * d - 1, d))        # remainder d - 1
    for n, d in cases:
        assert arith.div_newton(n, d) == divmod(n, d), (n.bit_length(), d.bit_length())


def test_pow10(arith):
    for e in [0, 1, 2, 9, 27, 28, 29, 31, 32, 33, 64, 100, 1000, 12345, 100000, 262143]:
        assert arith.pow10_exact(e) == 10 ** e, e


def test_to_decimal(arith):
    rng = random.Random(7)
    vals = [0, 1, 9, 10, 99, 10 ** 9 - 1, 10 ** 9, 10 ** 18, 2 ** 64 - 1, 2 ** 64, 10 ** 5000 + 1,
            2 ** 100000, 3 ** 40000]
    for k in [575, 576, 577, 1151, 1152, 1153, 2304, 4609, 9216, 36865]:
        vals += [10 ** k - 1, 10 ** k, 10 ** k + 1]
    for nl in [1, 2, 3, 19, 60, 61, 62, 64, 65, 200, 1000, 3000, 10000, 40000]:
        vals.append(_rand(rng, nl))
    for v in vals:
        assert arith.to_decimal(v) == str(v), v.bit_length()


def test_to_decimal_buffer_too_small(arith, engine):
    # the digits come from the device straight into the caller's buffer: a
    # buffer without room reports the digit count and GBNTT_ERR_SIZE and is
    # left untouched beyond its size
    import ctypes
    import numpy as np
    v = 3 ** 20000 + 12345
    want = str(v)
    a = np.frombuffer(v.to_bytes((v.bit_length() + 31) // 32 * 4, "little"), dtype=np.uint32).copy()
    lib = engine.lib()
    for cap in (1, 2, len(want), len(want) + 1):
        buf = ctypes.create_string_buffer(b"\x7f" * (cap + 8), cap + 8)
        n = ctypes.c_size_t(0)
        rc = lib.gbntt_to_decimal_u32(buf, cap, ctypes.byref(n), a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                      len(a))
        if cap >= len(want) + 1:
            assert rc == 0 and n.value == len(want) and buf.raw[:len(want)].decode() == want and buf.raw[len(want)] == 0
        else:
            assert rc == (5 if cap < 2 else 2), (cap, rc)   # GBNTT_ERR_ARG below 2 bytes, else GBNTT_ERR_SIZE
            if cap >= 2:
                assert n.value == len(want)
        assert buf.raw[cap:] == b"\x7f" * 8, cap


@pytest.mark.parametrize("top", ["0", "1", "4", "6", "7", "9", "11", "12"])
def test_to_decimal_block_levels(arith, top, monkeypatch):
    # The levels at and below GBNTT_DEC_TOP are split in shared memory by
    # Barrett steps against 10^(9 2^j); values at the level boundaries
    # (10^(9 2^k) +- 1), all-ones limbs (long carry and borrow chains) and
    # multiples of the divisors (remainders of zero) at every split.
    monkeypatch.setenv("GBNTT_DEC_TOP", top)
    rng = random.Random(int(top) + 100)
    vals = [1, 10 ** 9 - 1, 10 ** 18 - 1, 10 ** 18, 2 ** 64 - 1]
    for k in [9 << 1, 9 << 4, 9 << 7, 9 << 11, 9 << 12]:
        vals += [10 ** k - 1, 10 ** k, 10 ** k + 1, 10 ** k - 10 ** (k // 2), 7 * 10 ** (k - 1)]
    for nl in [2, 4, 8, 15, 30, 60, 120, 240, 479, 957, 1914, 3828, 3829, 7654]:
        vals.append((1 << (32 * nl)) - 1)
        vals.append(_rand(rng, nl))
    for v in vals:
        assert arith.to_decimal(v) == str(v), (top, v.bit_length())


@pytest.mark.parametrize("derive,wrap,short", [("0", "0", "0"), ("0", "1", "1"), ("1", "0", "1"), ("1", "1", "0"),
                                               ("1", "1", "1")])
def test_to_decimal_reciprocals(arith, derive, wrap, short, monkeypatch):
    # Levels above the block kernel divide by reciprocals of 10^(9 2^j),
    # each from its own Newton iteration (0) or derived from the level
    # above's (1), with remainders from full or cyclic products, and the top
    # level's reciprocal short (from the squared one of the level below) or
    # full; low tops put many levels on that path. 10^110000 + 7 needs a top
    # reciprocal of 3766 limbs, at the limit (3824) of the short form;
    # 10^147000 - 3 more than it can give (full-length fallback).
    monkeypatch.setenv("GBNTT_E_DERIVE_RECIP", derive)
    monkeypatch.setenv("GBNTT_E_WRAP", wrap)
    monkeypatch.setenv("GBNTT_E_SHORT_TOP", short)
    rng = random.Random(31)
    vals = [_rand(rng, 9000), (1 << (32 * 9000)) - 1, 10 ** 80000 - 1, 10 ** 73728, 10 ** 73728 - 1,
            10 ** 110000 + 7, 10 ** 147000 - 3]
    for top in ["2", "5", "11"]:
        monkeypatch.setenv("GBNTT_DEC_TOP", top)
        for v in vals:
            assert arith.to_decimal(v) == str(v), (derive, wrap, short, top, v.bit_length())


def test_compute_e_small(arith, e_gold):
    head = e_gold["1000"]["head"]
    for D in [1, 2, 3, 5, 10, 39]:
        assert arith.compute_e(D) == head[:D + 1], D


@pytest.mark.parametrize("D", [1000, 10000, 100000, 1000000])
def test_compute_e_matches_reference(arith, engine, e_gold, D):
    s = arith.compute_e(D)
    g = e_gold[str(D)]
    assert s[:40] == g["head"] and s[-40:] == g["tail"]
    assert hashlib.sha256(s.encode()).hexdigest() == g["sha256"]
    assert engine.device_errors() == 0


def test_compute_e_against_oracle_odd_sizes(arith):
    # sizes around the printed decimal pieces (288 digits) and level
    # boundaries (9 2^j digits)
    for D in [287, 288, 289, 575, 576, 577, 1152, 1153, 4608, 4609, 7777]:
        assert arith.compute_e(D) == eo.e_string(D), D


def test_compute_e_keeps_engine_and_reports_phases(arith, engine):
    s, ph = arith.compute_e(5000, phases=True)
    assert engine.is_ready() and engine.lib().gbntt_max_log() == 24
    assert len(ph) == 5 and all(p >= 0 for p in ph) and ph[4] >= max(ph[:4])
    assert s == arith.compute_e(5000)


def test_compute_e_1e7_matches_reference(arith, engine, e_gold):
    s = arith.compute_e(10 ** 7)
    g = e_gold["10000000"]
    assert s[-40:] == g["tail"]
    assert hashlib.sha256(s.encode()).hexdigest() == g["sha256"]
    assert engine.device_errors() == 0


def _run(body, timeout=900):
    r = subprocess.run([sys.executable, "-c", textwrap.dedent(body) % ROOT], capture_output=True, text=True,
                       timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_compute_e_initialises_its_own_engine_and_refuses_a_small_one():
    out = _run("""
        import json, sys
        sys.path.insert(0, %r)
        import cryptography_gb300 as g
        from cryptography_gb300 import arith
        s1 = arith.compute_e(2000)
        ready_after = g.is_ready()
        g.init(8)
        try:
            arith.compute_e(10 ** 6)
            rc = 0
        except g.EngineError as e:
            rc = e.code
        print(json.dumps([s1[:12], ready_after, rc, g.is_ready()]))
    """)
    assert out == ["2.7182818284", False, 2, True]


def test_compute_e_1e8_matches_reference(e_gold):
    g = e_gold.get("100000000")
    if g is None:
        pytest.skip("no 10^8 reference digits recorded")
    out = _run("""
        import hashlib, json, sys
        sys.path.insert(0, %r)
        from cryptography_gb300 import arith
        s, ph = arith.compute_e(10 ** 8, phases=True)
        print(json.dumps([hashlib.sha256(s.encode()).hexdigest(), s[:40], s[-40:], ph]))
    """)
    assert out[1] == g["head"] and out[2] == g["tail"]
    assert out[0] == g["sha256"]
