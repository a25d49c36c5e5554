"""Host-side pieces of libfactsieve.so (no GPU): exported symbols, power table,
setup plan, CPU factor checks, post-processing, capacity bounds."""
import math
import os
import random
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(fslib):
    import ctypes
    hdr = open(os.path.join(ROOT, "include", "factsieve.h")).read()
    names = sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(fs_\w+)\s*\(", hdr, re.M)))
    assert len(names) >= 30
    raw = ctypes.CDLL(fslib.LIB_PATH)
    missing = [n for n in names if not hasattr(raw, n)]
    assert not missing, missing


def test_power_table_equals_oracle(fslib, orc):
    for n in [127, 1000, 54_321, 100_000, 1_000_000]:
        a = fslib.power_table(n)
        b = orc.power_table(n)
        for x, y in zip(a, b):
            assert x.tolist() == y.tolist(), n


@pytest.mark.parametrize("n,chunks", [(127, 1), (1000, 1), (4999, 1), (4999, 3), (20_000, 7), (1, 1), (2, 1), (3, 1),
                                     (4, 1), (5, 2), (6, 1), (7, 3), (8, 1)])
def test_setup_plan_multiplies_to_factorial(fslib, n, chunks):
    """Horner over each chunk's layers (square, double, multiply words) multiplies to
    exactly n!, and each chunk's deficit counts one R^-1 per word, doubled by
    every later squaring -- the bookkeeping the GPU's final correction relies on."""
    words, layers, deficit = fslib.setup_plan(n, chunks)
    bounds, deficits = fslib.setup_plan_chunks(n, chunks)
    total = 1
    for c in range(chunks):
        x, d = 1, 0
        for li in range(int(bounds[c]), int(bounds[c + 1])):
            b, e, dbl, _ = layers[li].tolist()
            if li != bounds[c]:
                x *= x
                d *= 2
            if dbl:
                x *= 2
            for w in words[b:e].tolist():
                assert 1 < w < 2**64
                x *= w
                d += 1
        assert d == int(deficits[c])
        total *= x
    assert total == math.factorial(n)
    assert deficit == int(deficits.sum())


def _bfd_words(primes):
    """Best fit decreasing in plain Python: each word starts from the largest
    prime left and takes the largest prime that still fits below 2^64."""
    import bisect
    rem = sorted(primes)
    out = []
    while rem:
        w = rem.pop()
        while rem:
            i = bisect.bisect_right(rem, ((1 << 64) - 1) // w)
            if i == 0:
                break
            w *= rem.pop(i - 1)
        out.append(w)
    return out


@pytest.mark.parametrize("n", [1000, 54_321, 100_000])
def test_setup_plan_layers_are_packed_best_fit_decreasing(fslib, n):
    """Each layer's words are the odd primes whose Legendre exponent has that
    bit set, packed largest first, each word taking the largest prime that
    still fits (pack_layer, fs_host.cpp): the same words as a plain restatement,
    and never more than packing the ascending list in order."""
    words, layers, _ = fslib.setup_plan(n)
    primes = [q for q in range(3, n + 1, 2) if all(q % d for d in range(3, math.isqrt(q) + 1, 2))]
    exps = {q: sum(n // q**k for k in range(1, 64) if q**k <= n) for q in primes}
    nbits = len(layers)
    seq_total = 0
    for li in range(nbits):
        b = nbits - 1 - li                       # layers run from the top bit down
        lq = [q for q in primes if (exps[q] >> b) & 1]
        lo, hi = int(layers[li][0]), int(layers[li][1])
        assert words[lo:hi].tolist() == _bfd_words(lq), (n, b)
        w, cnt = 1, 0
        for q in lq:                             # ascending, in order
            if w * q >= 1 << 64:
                cnt, w = cnt + 1, q
            else:
                w *= q
        seq_total += cnt + (w != 1)
    assert len(words) <= seq_total
    bound = {1000: 1.0, 54_321: 0.97, 100_000: 0.92}[n]   # 4.2 % and 9.7 % fewer words at the larger n
    assert len(words) <= bound * seq_total


def test_setup_plan_is_shorter_than_reference_table(fslib):
    """The bit-layered plan needs fewer Montgomery products per candidate than the
    reference's table walk (setup.cl:56-102) -- the point of the rewrite."""
    for n in [100_000, 1_000_000]:
        words, layers, _ = fslib.setup_plan(n)
        tp, te, tb = fslib.power_table(n)
        ref = int(max(int(te[0]), 1).bit_length() - 1)
        for e in te[1:].tolist():
            ref += 2 + ((e.bit_length() - 1) + (bin(e).count("1") - 1) if e > 1 else 0)
        ours = len(words) + len(layers)
        assert ours * 2.5 < ref, (n, ours, ref)


def test_is_prime_and_verify_match_oracle(fslib, orc):
    rng = random.Random(3)
    from test_oracle import SPSP2
    nums = SPSP2 + [127, 65537, 1_000_000_007, (1 << 61) - 1, (1 << 64) - 59] + \
        [rng.randrange(3, 1 << 64) | 1 for _ in range(2000)]
    for n in nums:
        assert fslib.is_prime(n) == orc.is_prime(n), n
    for _ in range(60):
        p = rng.randrange(200, 1 << 63) | 1
        n = rng.randrange(127, 3000)
        for c in (-1, 1):
            assert fslib.verify_factor(p, n, c) == orc.verify(p, n, c), (p, n, c)


def test_verify_accepts_known_factors(fslib, orc):
    cand = orc.candidates(127, 2500)
    hits = orc.sieve_list(cand, 127, 2500)["hits"]
    assert len(hits) > 50
    for p, nc in zip(hits["p"].tolist(), hits["nc"].tolist()):
        assert fslib.verify_factor(p, abs(nc), -1 if nc < 0 else 1)
        assert not fslib.verify_factor(p, abs(nc), 1 if nc < 0 else -1) or p <= 3


def test_postprocess_equals_oracle(fslib, orc):
    """Sort, verify, 2-PRP filter and n + c checksum equal the oracle's restatement
    of getResults (cl_sieve.cpp:484-550), including a pseudoprime hit."""
    cand = np.concatenate([orc.candidates(127, 6000), np.array([2047, 3277], dtype=np.uint64)])
    hits = orc.sieve_list(cand, 127, 6000)["hits"]
    rng = np.random.default_rng(5)
    hits = hits[rng.permutation(len(hits))]
    kept_o, cs_o, disc_o = orc.postprocess(hits)
    kept_f, cs_f, disc_f = fslib.postprocess(hits, threads=4)
    assert cs_f == cs_o
    assert disc_f == disc_o
    assert kept_f[["p", "nc"]].tolist() == kept_o[["p", "nc"]].tolist()


def test_postprocess_rejects_a_bad_hit(fslib):
    bad = np.zeros(1, dtype=fslib.FACTOR_DTYPE)
    bad["p"] = 1_000_003
    bad["nc"] = 500
    with pytest.raises(fslib.FSError) as e:
        fslib.postprocess(bad)
    assert e.value.code == 7


@pytest.mark.parametrize("lo,hi", [(127, 128), (127, 100_000), (1_000_000, 2_000_000), (10**12, 10**12 + 10**6),
                                   ((1 << 63), (1 << 63) + 10**6), ((1 << 64) - 10**6, (1 << 64) - 1)])
def test_candidate_capacity_covers_oracle_count(fslib, orc, lo, hi):
    assert fslib.candidate_capacity(lo, hi) >= len(orc.candidates(lo, hi))


def test_context_needs_a_device(fslib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(fslib.FSError):
        fslib.Context(0)


def test_walk_step_selection_boundaries(fslib):
    """The launch-wide step the host proves valid for a p-segment (fs_walk_step)."""
    H64, T64, L96, C96, H96, H32, HM, C96H, HF, ANY = 4, 1, 2, 3, 5, 6, 7, 8, 9, 0
    HG, HGL, HG96, C96G = 10, 11, 12, 13
    ws = fslib.walk_step
    assert ws(10**12, 10**12 + 10**8, 200_000) == HF                       # config 2
    assert ws(10**12, 10**12 + 10**9, 200_000) == HF                       # config 2, whole range
    assert ws(1 << 63, (1 << 63) + 10**9, 1_010_000) == C96G               # config 3: float quotient
    assert ws(1 << 63, (1 << 63) + 10**9, 1_276_527) == C96H               # past its k_max bound
    assert ws(1 << 63, (1 << 63) + 10**9, 1 << 26) == C96                   # k_max >= 2^26 at p >= 2^63
    assert ws(10**6, 2 * 10**6, 2000) == H32                               # config 1: p < 2^31
    assert ws(127, 100_000, 1_000_000) == H32                              # self test 3 (p <= nmax)
    assert ws((1 << 31) - 1000, (1 << 31) + 1000, 2000) == ANY              # straddles 2^31
    assert ws((1 << 32) + 1, (1 << 32) + 1000, 2000) == HGL                 # 2^31 <= p, window s <= 32: float quotient
    assert ws((1 << 32) + 1, (1 << 32) + 1000, 1_276_527) == HM             # ... k_max past 46 k_max < 7 2^23: shifted window
    assert ws((1 << 32) + 1, (1 << 32) + 1000, 1 << 25) == ANY              # ... with k_max >= 2^25: generic
    assert ws(10**6, 2 * 10**6, 1 << 26) == ANY                             # k_max >= 2^26 at small p
    assert ws(1 << 36, (1 << 36) + 1000, 2000) == HGL
    assert ws((1 << 36) - 1000, (1 << 36) + 1000, 2000) == HGL              # no bound at 2^36 for the float quotient
    assert ws(1 << 36, (1 << 36) + 1000, 1 << 21) == H64                    # k_max past the float quotient's bound
    assert ws((1 << 36) - 1000, (1 << 36) + 1000, 1 << 21) == T64           # ... straddling 2^36: the step valid on both sides
    # float-quotient step: p >= 2^38, 19 kmax <= 2^23, 19 pmax kmax < 2^(bitlen(plo) + 23), p kmax <= 2^62
    assert ws(1 << 38, (1 << 38) + 1000, 2000) == HF
    assert ws((1 << 38) - 1000, (1 << 38) + 1000, 2000) == HGL             # straddles 2^38: window s = 26 on both sides
    assert ws(10**12, 10**12 + 30_000, 441_505) == HF                       # 19 kmax <= 2^23
    assert ws(10**12, 10**12 + 30_000, 441_506) == HG                       # k_max-aware window, s >= 32
    assert ws((1 << 39) + 1, (1 << 40) - 1, 441_505) == HF                  # 19 pmax kmax < 2^63
    assert ws((1 << 39) - 1000, (1 << 40) - 1, 441_505) == HG               # bitlen(plo) 39: z could reach 2^23 in HF's window
    assert ws((1 << 50) - 10_000, (1 << 50) + 1, 4096) == HF                # p kmax = 2^62 exactly
    assert ws((1 << 50) - 10_000, (1 << 50) + 2, 4096) == HG                # just above: t < 23/16 p k_max < 2^64 still
    assert ws((1 << 35) + 1, (1 << 35) + 1000, 1 << 25) == T64              # 2^33 < p < 2^36, k_max >= 2^25
    k = 1 << 20
    assert ws(1 << 40, (1 << 40) + 1, k) == HG                              # p kmax = 2^60
    assert ws((1 << 42) - 10, (1 << 42) + 1, k) == HG                       # p kmax = 2^62 exactly
    assert ws((1 << 44) + 1, (1 << 44) + 1000, k) == HG96                   # 23/16 p k_max >= 2^64: 96-bit t
    assert ws((1 << 42) - 10, (1 << 42) + 2, 1 << 21) == H96                # k_max past the bound: 96-bit, half-offset
    # HG needs 23/16 pmax k_max < 2^64 (t in 64 bits), HG96 p < 2^63 and s < 64
    kb = 1_276_526
    edge = ((1 << 68) - 1) // (23 * kb)                                     # last pmax with ceil(23 pmax kb / 16) < 2^64
    assert ws(edge - 1000, edge + 1, kb) == HG and ws(edge - 1000, edge + 2, kb) == HG96
    assert ws((1 << 63) - 10**6, (1 << 63) - 1, kb) == HG96 and ws((1 << 63) - 10**6, 1 << 63, kb) == HG96
    assert ws(1 << 63, (1 << 63) + 10**6, 1000) == C96G                     # p >= 2^63: the 96-bit canonical form
    assert ws((1 << 64) - 10**6, (1 << 64) - 1, kb) == C96G
    # the window shift on one side of 32: HGL while T = ceil(23 pmax k_max / 16) < 2^56
    # (s <= 32), HG while T(plo) >= 2^55 (s >= 32), neither across both
    T = lambda p: (23 * p * kb + 15) // 16
    last56, first55 = 39_268_312_544, 19_634_156_273
    assert T(last56) < 1 << 56 <= T(last56 + 1) and T(first55 - 1) < 1 << 55 <= T(first55)
    assert ws(last56 - 1000, last56 + 1, kb) == HGL and ws(last56 - 1000, last56 + 2, kb) == HG
    assert ws(first55, last56 + 10**6, kb) == HG
    assert ws(first55 - 1, last56 + 10**6, kb) == HM                       # s from 31 to 33: shifted window
    assert ws(10**13, 10**13 + 30_000, (1 << 26) - 1) == H96                # k_max past the float quotient's bound
    assert ws(10**13, 10**13 + 30_000, 1 << 26) == L96
    assert ws(10**13, 10**13 + 30_000, 1 << 28) == ANY                      # k_max >= 2^28: generic
    assert ws((1 << 63) - 1000, (1 << 63) + 1000, 5000) == ANY              # straddles 2^63
    assert ws(5, 5, 100) == ANY and ws(10**12, 10**12 + 5, 0) == ANY        # empty ranges


def test_setup_form_boundaries(fslib):
    """The setup folds its products modulo 2^63 + d exactly when every p of the
    segment is 2^63 + d with d < 2^30 (fs_setup_form)."""
    sf = fslib.setup_form
    assert sf(1 << 63, (1 << 63) + 10**9) == 1                             # config 3 (2^63 is even: d >= 1)
    assert sf(1 << 63, (1 << 63) + 10**8) == 1
    assert sf((1 << 63) + (1 << 30) - 1000, (1 << 63) + (1 << 30)) == 1    # d up to 2^30 - 1
    assert sf((1 << 63) + (1 << 30) - 1000, (1 << 63) + (1 << 30) + 1) == 0
    assert sf((1 << 63) - 1000, (1 << 63) + 1000) == 0                     # straddles 2^63
    assert sf(10**12, 10**12 + 10**9) == 0
    assert sf((1 << 63) + 5, (1 << 63) + 5) == 0                           # empty


def test_c_caller(fslib, tmp_path):
    """The header and library serve a plain C program (gcc, no C++ or Python in between)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / "c_abi_example")
    libdir = os.path.dirname(fslib.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_abi_example.c"), "-L", libdir, "-lfactsieve",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True, capture_output=True, text=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=60).stdout
    got = dict(line.split(" ", 1) for line in out.strip().splitlines())
    assert got["parse_p"] == "0 1000000000000" and got["parse_P"] == "0 1001000000000"
    assert got["parse_n"] == "0 100000" and got["bad_arg"] != "0"
    assert got["is_prime"] == "1 0"
    assert got["verify"] == "1 0 1"
    rc, kept, cs, disc, first = got["postprocess"].split()
    assert (rc, kept, disc, first) == ("0", "2", "0", "149")          # sorted by (p, |n|), both kept
    assert int(cs) == (25 - 1) + (169725 + 1)                          # checksum += n + c per kept factor
    assert int(got["capacity"]) == fslib.candidate_capacity(10**12, 10**12 + 10**8)
    assert got["walk_step"] == "9 6"
    assert got["strerror"].strip() == fslib.lib().fs_strerror(fslib.FS_E_OVERFLOW).decode()


def _f32(bits):
    import struct
    from fractions import Fraction
    return Fraction(struct.unpack("<f", struct.pack("<I", bits & 0xFFFFFFFF))[0])


def _halff_step(r, k, p, f):
    """Word-level restatement of halff_step (fs_arith.cuh) with exact rationals:
    z = (t's high word) >> (s - 32) read as the subnormal z 2^-149, one fma by
    m 2^(s-e) rounding down onto the subnormal grid."""
    from fractions import Fraction
    bl, s = p.bit_length(), f.bit_length() - 4
    e = bl + 23
    m = (1 << e) // p
    assert (1 << 23) <= m < (1 << 24)
    g = _f32(((s - e + 149) << 23) + m)
    assert g == Fraction(m, 1 << (e - s))
    t = r * k
    assert t < 1 << 64
    z = (t >> 32) >> (s - 32)
    assert z < 1 << 23
    assert _f32(z) == Fraction(z, 1 << 149)                  # exponent field 0: the subnormal z 2^-149
    prod = _f32(z) * g
    assert prod < Fraction(1, 1 << 126)                      # on the subnormal grid
    q = int(prod * (1 << 149))
    return (t + q * ((1 << 64) - p)) % (1 << 64)


def test_float_quotient_window_holds_where_the_host_selects_it(fslib):
    """Wherever fs_walk_step picks the float-quotient step, the step is exact and
    keeps r below (19/16) p < x + p, the bound the two-compare hit test needs.
    Checked for the least and largest p of each range, with the thread floor at
    the range's low end, over the last multipliers up to k_max."""
    import random
    rng = random.Random(3)
    n = 0
    while n < 40:
        bits = rng.randrange(38, 61)
        lo = rng.randrange(1 << bits, 1 << (bits + 1))
        w = rng.choice([1000, 10**6, 1 << (bits - 2)])
        kmax = rng.choice([rng.randrange(2, 441_506), 441_505])
        if fslib.walk_step(lo, lo + w, kmax) != 9:
            continue
        n += 1
        for p in (lo | 1, (lo + w - 1) | 1):
            if p >= lo + w:
                p -= 2
            r = p - 1
            for k in range(max(1, kmax - 150), kmax + 1):
                r2 = _halff_step(r, k, p, lo)
                assert r2 % p == (r * k) % p
                assert 16 * r2 < 19 * p
                r = r2


def _halfg_step(r, k, p, kmax, form):
    """Word-level restatement of the float-quotient steps with a k_max-aware
    window (make_halfg, fs_arith.cuh): s = bitlen(ceil(23 p kmax / 16)) - 24,
    z = floor(t / 2^s) read as the subnormal z 2^-149 (24 bits at most), one
    fma by m 2^(s-e) rounding down on the subnormal grid.  form: 10 HG, 11 HGL,
    12 HG96 (fs_walk_step's values)."""
    from fractions import Fraction
    T = (23 * p * kmax + 15) // 16
    s = T.bit_length() - 24
    assert (s >= 32) if form in (10, 12) else (s <= 32)
    bl = p.bit_length()
    e = bl + 23
    m = (1 << e) // p
    assert (1 << 23) <= m < (1 << 24)
    g = _f32(((s - e + 149) << 23) + m)
    assert g == Fraction(m, 1 << (e - s))
    t = r * k
    assert t < (1 << 64) if form in (10, 11) else t < (1 << 96)
    z = t >> s
    assert z < 1 << 24
    assert _f32(z) == Fraction(z, 1 << 149)                  # exponent field 0 or 1: spacing 2^-149
    prod = _f32(z) * g
    assert prod < Fraction(1, 1 << 125)
    q = int(prod * (1 << 149))
    assert q <= t // p
    return (t + q * ((1 << 64) - p)) % (1 << 64)


def test_kmax_window_float_quotient_holds_where_the_host_selects_it(fslib):
    """Wherever fs_walk_step picks one of the float-quotient steps with a
    k_max-aware window (10, 11, 12), each step is exact and keeps r below
    (23/16) p < x + p, for the least and largest p of the range over the last
    multipliers up to k_max, k_max up to the bound 46 k_max < 7 2^23."""
    import random
    rng = random.Random(5)
    seen = {10: 0, 11: 0, 12: 0}
    tries = 0
    while min(seen.values()) < 12:
        tries += 1
        assert tries < 200_000
        bits = rng.randrange(31, 63)
        lo = rng.randrange(1 << bits, 1 << (bits + 1))
        if lo >= 1 << 63:
            continue
        w = rng.choice([1000, 10**6, 1 << max(bits - 8, 10)])
        kmax = rng.choice([rng.randrange(441_506, 1_276_527), 1_276_526, rng.randrange(2, 441_506)])
        step = fslib.walk_step(lo, lo + w, kmax)
        if step not in seen:
            continue
        seen[step] += 1
        for p in (lo | 1, (lo + w - 1) | 1):
            if p >= lo + w:
                p -= 2
            r = p - 1
            for k in range(max(1, kmax - 120), kmax + 1):
                r2 = _halfg_step(r, k, p, kmax, step)
                assert r2 % p == (r * k) % p
                assert 16 * r2 < 23 * p
                r = r2
    # the corners: p just below 2^63 with k_max at the bound (96-bit t), and
    # the window shift on both sides of 32
    for lo, hi, kmax, want in [((1 << 63) - 10_001, (1 << 63) - 1, 1_276_526, 12),
                               ((1 << 31) + 1, (1 << 31) + 1001, 1_276_526, 11),
                               ((1 << 40) + 1, (1 << 40) + 1001, 1_276_526, 10)]:
        assert fslib.walk_step(lo, hi, kmax) == want
        p = (hi - 2) | 1
        r = p - 1
        for k in range(kmax - 200, kmax + 1):
            r2 = _halfg_step(r, k, p, kmax, want)
            assert r2 % p == (r * k) % p and 16 * r2 < 23 * p
            r = r2
    # beyond the k_max bound the steps are not chosen
    assert fslib.walk_step((1 << 40) + 1, (1 << 40) + 1001, 1_276_527) not in (10, 11, 12)


def _c96g_step(r, k, p, kmax):
    """Word-level restatement of the float-quotient step for p >= 2^63
    (canon96g_walk8x2, fs_arith.cuh) on a lazy residue of up to 65 bits:
    t = r k, s = bitlen(ceil(23 p kmax / 16)) - 24, z = t >> s read as the
    subnormal z 2^-149, one round-down fma by g = m 2^(s-87), m = floor(2^87 / p);
    r' = t - q p, exact."""
    from fractions import Fraction
    assert p >> 63
    T = (23 * p * kmax + 15) // 16
    s = T.bit_length() - 24
    assert 32 <= s < 64
    m = (1 << 87) // p
    assert (1 << 23) <= m < (1 << 24)
    g = _f32(((s - 87 + 149) << 23) + m)
    assert g == Fraction(m, 1 << (87 - s))
    t = r * k
    assert t < 1 << 96
    z = t >> s
    assert z < 1 << 24 and z == ((t >> 32) >> (s - 32)) & 0xFFFFFFFF    # the funnel shift of t's upper words
    q = int(_f32(z) * g * (1 << 149))
    assert q <= t // p
    return t - q * p


def test_float_quotient_for_p_above_2_63_keeps_its_bound(fslib):
    """Wherever fs_walk_step picks the float-quotient 96-bit step for p >= 2^63
    (13), each step is exact, never negative, and keeps the lazy residue below
    (23/16) p (65 bits) over the last multipliers up to k_max, at the bound."""
    import random
    rng = random.Random(13)
    for _ in range(40):
        lo = rng.choice([(1 << 63) + rng.randrange(1, 1 << 30), rng.randrange(1 << 63, (1 << 64) - 10**6),
                         (1 << 64) - rng.randrange(10**6, 10**7)])
        kmax = rng.choice([1_276_526, rng.randrange(2, 1_276_527), rng.randrange(1_000_000, 1_276_527)])
        hi = lo + 1000
        assert fslib.walk_step(lo, hi, kmax) == 13
        for p in ((lo | 1), (hi - 2) | 1):
            r = p - 1
            for k in range(max(1, kmax - 120), kmax + 1):
                r2 = _c96g_step(r, k, p, kmax)
                assert r2 >= 0 and r2 % p == (r * k) % p and 16 * r2 < 23 * p
                r = r2


def _pm_mul(a, b, p):
    """Word-level restatement of pm_mul (fs_arith.cuh): fold 2^64 = -2d modulo
    p = 2^63 + d twice, add p - 2d on a carry out."""
    M = (1 << 64) - 1
    e = 2 * (p - (1 << 63))
    x = a * b
    x0, x1 = x & M, x >> 64
    w = e * x1
    w0, w1 = w & M, w >> 64
    assert w1 < e
    u, borrow = (x0 - w0) & M, int(x0 < w0)
    v = e * (w1 + borrow)
    assert v < 1 << 62
    y = u + v
    if y >> 64:
        y = (y & M) + (p - e)
        assert y < 1 << 64
    return y


def test_folded_product_is_exact_where_the_host_selects_it(fslib):
    """Wherever fs_setup_form selects the folding product, it is congruent to a b
    for any 64-bit inputs and stays below 2^64, over chains as the setup runs them."""
    import random
    rng = random.Random(4)
    for _ in range(30):
        d = rng.choice([1, rng.randrange(1, 1 << 30), (1 << 30) - 1]) | 1
        p = (1 << 63) + d
        assert fslib.setup_form(p, p + 1) == 1
        x, ex = 1, 1
        for _ in range(200):
            w = rng.choice([rng.randrange(1 << 64), (1 << 64) - 1, 2, p, p - 1])
            x = _pm_mul(x, w, p)
            ex = ex * w % p
            assert x < 1 << 64 and x % p == ex
        assert _pm_mul((1 << 64) - 1, (1 << 64) - 1, p) % p == ((1 << 64) - 1) ** 2 % p
