"""CPU tests of the compute_e oracle: pinned to the reference's own printed
digits (tests/golden/e_digits.json, made by make_e_golden.py from the
reference's compiled host compute_e), and the library's host-only term
count against the reference formula."""
import hashlib
import json
import os

import pytest

from oracle import e_oracle as eo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "e_digits.json")


@pytest.fixture(scope="module")
def e_gold():
    with open(GOLD) as f:
        return json.load(f)


@pytest.mark.parametrize("D", [1000, 10000, 100000])
def test_oracle_matches_reference_digits(e_gold, D):
    s = eo.e_string(D)
    g = e_gold[str(D)]
    assert s[:40] == g["head"] and s[-40:] == g["tail"]
    assert hashlib.sha256(s.encode()).hexdigest() == g["sha256"]


def test_golden_prefixes_agree(e_gold):
    # longer runs of the reference repeat the shorter ones' digits
    heads = {g["head"] for g in e_gold.values()}
    assert len(heads) == 1


def test_binary_split_shapes_agree():
    for a, b in [(1, 2), (1, 3), (5, 6), (7, 7), (9, 4), (1, 100), (17, 1000)]:
        assert eo.binary_split(a, b) == eo.binary_split_seq(a, b), (a, b)


def test_split_terms_reference_values():
    # K for d = 10^8 (+20 guard digits) as the reference's run reports it
    assert eo.split_terms_needed(10 ** 8 + 20) == 15585119


def test_library_term_count_matches_formula(built_lib):
    for n in [1, 2, 5, 21, 100, 1020, 10 ** 5 + 20, 10 ** 6 + 20, 10 ** 7 + 20, 10 ** 8 + 20, 3 * 10 ** 9]:
        assert built_lib.gbntt_split_terms_needed(n) == eo.split_terms_needed(n), n


def test_library_e_required_log(built_lib):
    from cryptography_gb300 import arith
    logs = [arith.e_required_log(d) for d in (1, 1000, 10 ** 6, 10 ** 8)]
    assert logs == sorted(logs) and logs[-1] <= 26
    assert built_lib.gbntt_e_required_log(0) < 0


@pytest.mark.parametrize("D", [1000, 100000, 1000000])
def test_gmp_port_matches_reference_digits(e_gold, D):
    s, t = eo.gmp_e_string(D)
    assert hashlib.sha256(s.encode()).hexdigest() == e_gold[str(D)]["sha256"]
    assert t >= 0
