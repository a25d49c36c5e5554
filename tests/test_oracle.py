"""The CPU oracle against the reference: self-test goldens, the reference's own
CPU arithmetic (verifyprime.c), and the constant tables of its kernels."""
import json
import os
import random
import re

import numpy as np
import pytest

from conftest import REFERENCE

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SELFTEST = {
    1: (100_000_000, 101_000_000, 1_000_000, 2_000_000, 1071, 54211, 0x000004F4F744CA97),
    2: (1_000_000_000_000, 1_000_010_000_000, 10_000, 2_000_000, 3, 361727, 0x05052A2D65F3D735),
    3: (127, 100_000, 127, 1_000_000, 42770, 9566, 0x0000000065C074F0),
    4: (2_000_000_000_000, 2_000_010_000_000, 2_000_000, 6_000_000, 3, 352866, 0x09C9742A908451EB),
    5: (1_000_000_000_000, 1_000_001_000_000, 100_000_000, 110_000_000, 3, 36249, 0x0081056DC98DA092),
}

# base-2 strong pseudoprimes (composite, pass SPRP-2); the generator must keep
# those without a factor <= 113 and the host filter must drop them
SPSP2 = [2047, 3277, 4033, 4681, 8321, 15841, 29341, 42799, 49141, 52633, 65281, 74665, 80581, 85489,
         88357, 90751, 104653, 130561, 196093, 220729, 233017, 252601, 253241, 256999, 271951, 280601,
         314821, 357761, 390937, 458989, 476971, 486737, 3215031751, 3825123056546413051]


def _small_factor(n):
    return any(n % q == 0 for q in [2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67,
                                    71, 73, 79, 83, 89, 97, 101, 103, 107, 109, 113])


def test_selftest3_matches_reference_golden(orc):
    pmin, pmax, nmin, nmax, fc, pc, cs = SELFTEST[3]
    r = orc.run(pmin, pmax, nmin, nmax)
    assert (r["factorcount"], r["primecount"], r["checksum"]) == (fc, pc, cs)
    assert r["nvalidfail"] == 0


@pytest.mark.slow
@pytest.mark.parametrize("case", [1, 2, 4, 5])
def test_long_selftests_match_reference_golden(orc, case):
    pmin, pmax, nmin, nmax, fc, pc, cs = SELFTEST[case]
    r = orc.run(pmin, pmax, nmin, nmax)
    assert (r["factorcount"], r["primecount"], r["checksum"]) == (fc, pc, cs)


def test_committed_selftest_fixtures_carry_reference_goldens():
    """Fixtures made by make_golden.py for the self-test ranges hold the reference triples."""
    seen = 0
    for case, (pmin, pmax, nmin, nmax, fc, pc, cs) in SELFTEST.items():
        path = os.path.join(GOLD, f"run_selftest{case}.json")
        if not os.path.exists(path):
            continue
        g = json.load(open(path))
        assert (g["pmin"], g["pmax"], g["nmin"], g["nmax"]) == (pmin, pmax, nmin, nmax)
        assert (g["factorcount"], g["primecount"], g["checksum"]) == (fc, pc, f"{cs:016X}")
        seen += 1
    assert seen >= 1


def test_config1_fixture_reproduces(orc):
    g = json.load(open(os.path.join(GOLD, "run_config1.json")))
    r = orc.run(g["pmin"], g["pmax"], g["nmin"], g["nmax"])
    assert r["primecount"] == g["primecount"] == 70456
    assert f"{r['checksum']:016X}" == g["checksum"] == "000000188AA0823D"
    assert r["factorcount"] == g["factorcount"] == 106


@pytest.mark.parametrize("lo,hi", [(127, 30_000), (1_000_000, 1_050_000), ((1 << 32) - 9_000, (1 << 32) + 9_000),
                                   ((1 << 63) - 2_000, (1 << 63) + 2_000), ((1 << 64) - 5_000, (1 << 64) - 1),
                                   (129, 131), (999_999_999_989, 1_000_000_000_100)])
def test_candidate_walk_equals_definition(orc, lo, hi):
    """The 60-integer wheel walk of getsegprimes equals 'odd, no factor <= 113, SPRP-2'."""
    assert orc.candidates(lo, hi).tolist() == orc.candidates(lo, hi, naive=True).tolist()


def test_known_pseudoprimes(orc):
    for n in SPSP2:
        assert orc.sprp2(n), n
        assert not orc.is_prime(n), n
        got = orc.candidates(n - 10, n + 10).tolist()
        assert (n in got) == (not _small_factor(n)), n


def _reference_masks():
    path = os.path.join(REFERENCE, "kernels", "getsegprimes.cl")
    if not os.path.exists(path):
        pytest.skip("reference tree not present")
    txt = open(path).read()
    out = {}
    for m in re.finditer(r"__constant uint p(\d+)\[\d+\] = \{([^}]*)\}", txt):
        out[int(m.group(1))] = [int(x) for x in m.group(2).replace(" ", "").split(",")]
    return out


def test_small_prime_masks_equal_reference_tables(orc):
    """The reference's p7..p113 constant tables (getsegprimes.cl:116-168) are exactly
    'bit i set iff q | P + 2i' for P % q == r; the oracle and the GPU generate them."""
    ref = _reference_masks()
    assert sorted(ref) == [7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89,
                           97, 101, 103, 107, 109, 113]
    for q, tab in ref.items():
        assert len(tab) == q
        assert tab == [orc.small_mask(q, r) for r in range(q)], q


def _reference_wheel_walk(start):
    """cl_sieve.cpp:360-419 restated step by step (mod-6 walk forward, anchor on a
    multiple of 5, walk the mod-30 gaps back)."""
    wheel = [4, 2, 4, 2, 4, 6, 2, 6]
    k = start // 6
    i = 1
    n = k * 6 - 1
    while n < start or n % 5 == 0:
        if i:
            i = 0
            n += 2
        else:
            i = 1
            n += 4
    start = n
    idx = -1
    while idx < 0:
        if i:
            n += 2
            i = 0
            if n % 5 == 0:
                n -= 2
                idx = 5
        else:
            n += 4
            i = 1
            if n % 5 == 0:
                n -= 4
                idx = 7
    while n != start:
        idx -= 1
        if idx < 0:
            idx = 7
        n -= wheel[idx]
    return start, idx


def test_wheel_offset_matches_reference_walk(orc, fslib):
    rng = random.Random(7)
    starts = [127, 128, 130, 131, 150, 1_000_000, 1 << 40, (1 << 63) + 1] + [rng.randrange(127, 1 << 62)
                                                                             for _ in range(300)]
    for s in starts:
        want = _reference_wheel_walk(s)
        assert orc.find_wheel_offset(s) == want, s
        assert fslib.find_wheel_offset(s) == want, s


def test_oracle_arithmetic_equals_reference_verifyprime(orc, refmath):
    """oracle m_mul / add / invert / isPrime / verify against the reference's own
    verifyprime.c compiled from the reference tree."""
    rng = random.Random(11)
    for _ in range(3000):
        p = rng.randrange(3, 1 << 64) | 1
        q = refmath.invert(p)
        assert orc.invert(p) == q
        a, b = rng.randrange(p), rng.randrange(p)
        assert orc.mmul(a, b, p, q) == refmath.m_mul(a, b, p, q)
        assert orc.lib().oracle_madd(a, b, p) == refmath.add(a, b, p)
    for n in SPSP2 + [127, 131, 65537, 1_000_000_007, (1 << 61) - 1, (1 << 64) - 59]:
        assert orc.is_prime(n) == bool(refmath.isPrime(n)), n
    for _ in range(40):
        p = rng.randrange(1000, 1 << 63) | 1
        n = rng.randrange(40, 4000)
        for c in (-1, 1):
            assert orc.verify(p, n, c) == bool(refmath.verify(p, n, c))


def test_oracle_hits_verify_with_reference(orc, refmath):
    """Every hit the oracle finds on a dense range passes the reference's verify()."""
    cand = orc.candidates(127, 3000)
    out = orc.sieve_list(cand, 127, 3000)
    assert len(out["hits"]) > 100
    for p, nc in zip(out["hits"]["p"].tolist(), out["hits"]["nc"].tolist()):
        assert refmath.verify(p, abs(nc), -1 if nc < 0 else 1)


@pytest.mark.parametrize("nmin,nmax", [(34, 400), (127, 900), (300, 301)])
def test_exact_definition_equals_restatement_where_the_reference_is_valid(orc, nmin, nmax):
    """From nmin = 34 up the pure-Python definition and the reference restatement agree bit for bit."""
    e = orc.exact_small(127, 60_000, nmin, nmax)
    r = orc.run(127, 60_000, nmin, nmax)
    assert r["status"] == 0
    assert (e["primecount"], e["raw_sum"], e["checksum"], e["factorcount"]) == \
        (r["primecount"], r["raw_sum"], r["checksum"], r["factorcount"])
    assert e["factors"] == [(int(p), int(nc)) for p, nc in zip(r["factors"]["p"], r["factors"]["nc"])]


def test_reference_is_invalid_below_nmin_34(orc):
    """The domain edge the GPU path treats exactly: nmin 2 and 3 start from a wrong
    residue in the reference (getPower's curBit for exponent 1) and hits with
    n < 34 fail its verifier, which starts from 34!."""
    e = orc.exact_small(127, 60_000, 3, 400)
    r = orc.run(127, 60_000, 3, 400)
    assert r["raw_sum"] != e["raw_sum"]
    assert orc.run(127, 60_000, 20, 400)["status"] == -1          # a true factor with n < 34 rejected
    assert orc.exact_small(127, 60_000, 20, 400)["raw_sum"] == orc.run(127, 60_000, 20, 400)["raw_sum"]
    import math
    assert (math.factorial(25) - 1) % 149 == 0 and not orc.verify(149, 25, -1)   # 149 | 25! - 1, rejected
