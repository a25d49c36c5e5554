"""GPU parity: the CUDA path through the C ABI against the oracle and the goldens.

Every comparison is exact (integer work): candidate sets, residues, hit
lists, checksums and prime counts must be bit-identical.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# The reference's own self-test goldens (cl_sieve.cpp:1283-1364):
# (pmin, pmax, nmin, nmax, factorcount, primecount, checksum)
SELFTEST = {
    1: (100_000_000, 101_000_000, 1_000_000, 2_000_000, 1071, 54211, 0x000004F4F744CA97),
    2: (1_000_000_000_000, 1_000_010_000_000, 10_000, 2_000_000, 3, 361727, 0x05052A2D65F3D735),
    3: (127, 100_000, 127, 1_000_000, 42770, 9566, 0x0000000065C074F0),
    4: (2_000_000_000_000, 2_000_010_000_000, 2_000_000, 6_000_000, 3, 352866, 0x09C9742A908451EB),
    5: (1_000_000_000_000, 1_000_001_000_000, 100_000_000, 110_000_000, 3, 36249, 0x0081056DC98DA092),
}


def _torch():
    import torch
    return torch


def _dev_buffers(n_cand, n_hits=1 << 16):
    torch = _torch()
    cand = torch.zeros(max(n_cand, 1), dtype=torch.int64, device="cuda")
    import factsieve_gb300 as fs
    res = torch.zeros(fs.walk_state_words(max(n_cand, 1)), dtype=torch.int64, device="cuda")
    hits = torch.zeros(max(n_hits, 1) * 2, dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")   # 32-byte fs_counters
    # the library's stream does not wait for torch's: the zero fills must be done first
    torch.cuda.synchronize()
    return cand, res, hits, ctr


def _u64(t):
    return t.cpu().numpy().view(np.uint64)


def _counters(ctr):
    import factsieve_gb300 as fs
    return np.frombuffer(ctr.cpu().numpy().tobytes(), dtype=fs.COUNTERS_DTYPE)[0]


def _hits_array(hits, n):
    import factsieve_gb300 as fs
    raw = hits.cpu().numpy().tobytes()
    return np.frombuffer(raw, dtype=fs.FACTOR_DTYPE, count=n).copy()


def _sorted_hits(h):
    return sorted(zip(h["p"].tolist(), h["nc"].tolist()))


@pytest.mark.parametrize("idx", range(10))
def test_candidates_match_oracle(ctx, idx):
    with open(os.path.join(GOLD, "candidates_small.json")) as fh:
        case = json.load(fh)[idx]
    lo, hi, want = case["low"], case["high"], case["candidates"]
    import factsieve_gb300 as fs
    cap = fs.candidate_capacity(lo, hi)
    cand, _, _, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.synchronize()
    c = _counters(ctr)
    got = np.sort(_u64(cand)[: c["ncand"]])
    assert c["ncand"] == len(want)
    assert got.tolist() == sorted(want)


def _golden(name):
    path = os.path.join(GOLD, f"run_{name}.json")
    if not os.path.exists(path):
        pytest.skip(f"fixture {name} not generated")
    with open(path) as fh:
        return json.load(fh)


@pytest.mark.parametrize("name", ["config1", "selftest3", "wilson_small", "top_of_u64", "near_2p32",
                                  "near_2p62", "single_n", "nmin_eq_nmax"])
def test_search_matches_golden(ctx, name):
    g = _golden(name)
    r = ctx.sieve(g["pmin"], g["pmax"], g["nmin"], g["nmax"], threads=8)
    assert r.primecount == g["primecount"]
    assert f"{r.raw_sum:016X}" == g["raw_sum"]
    assert r.nhits == g["nhits"]
    assert f"{r.checksum:016X}" == g["checksum"]
    assert r.factorcount == g["factorcount"]
    if "factors" in g:
        assert r.lines() == g["factors"]


@pytest.mark.parametrize("case", [1, 2, 4, 5])
def test_reference_selftest(ctx, case):
    pmin, pmax, nmin, nmax, fc, pc, cs = SELFTEST[case]
    r = ctx.sieve(pmin, pmax, nmin, nmax, threads=16)
    assert (r.factorcount, r.primecount, r.checksum) == (fc, pc, cs)


def test_stage_api_matches_oracle(ctx, orc):
    """getsegprimes -> setup -> iterate (two chunks) -> check against the oracle."""
    lo, hi, nmin, nmax = 2_000_003, 2_060_000, 3000, 4500
    want_c = orc.candidates(lo, hi)
    import factsieve_gb300 as fs
    cap = fs.candidate_capacity(lo, hi)
    cand, res, hits, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), nmin, res.data_ptr())
    ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmin, 3700, hits.data_ptr(), 1 << 16)
    ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), 3700, nmax, hits.data_ptr(), 1 << 16)
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmax)
    ctx.synchronize()
    c = _counters(ctr)
    n = int(c["ncand"])
    got_c = _u64(cand)[:n]
    order = np.argsort(got_c)
    assert got_c[order].tolist() == want_c.tolist()
    want = orc.sieve_list(want_c, nmin, nmax, want_residues=True)
    assert _u64(res)[:n][order].tolist() == want["s6"].tolist()
    assert int(c["raw_sum"]) == want["raw_sum"]
    assert int(c["primecount"]) == n
    assert int(c["flags"]) == 0
    assert _sorted_hits(_hits_array(hits, int(c["nhits"]))) == _sorted_hits(want["hits"])


@pytest.mark.parametrize("nmin", [127, 1000, 54_321, 1_000_000])
def test_setup_residue_matches_oracle(ctx, orc, nmin):
    """nmin! * 2^64 mod p from the bit-layered table equals the reference table's."""
    import factsieve_gb300 as fs
    lo = max(nmin, 1_000_000_007)
    hi = lo + 40_000
    want_c = orc.candidates(lo, hi)
    table = orc.power_table(nmin)
    cap = fs.candidate_capacity(lo, hi)
    cand, res, _, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), nmin, res.data_ptr())
    ctx.synchronize()
    n = int(_counters(ctr)["ncand"])
    got_c = _u64(cand)[:n]
    order = np.argsort(got_c)
    got = _u64(res)[:n][order]
    want = [orc.setup(int(p), table) for p in want_c[:200]]
    assert got[:200].tolist() == want


@pytest.mark.parametrize("nmin", [127, 5000, 1_000_000, 20_000_000])
def test_table_check_agrees(ctx, nmin):
    import factsieve_gb300 as fs
    lo, hi = 1_000_000_000_039, 1_000_000_100_000
    cap = fs.candidate_capacity(lo, hi)
    cand, _, _, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    direct, table = ctx.table_check(cand.data_ptr(), ctr.data_ptr(), nmin)
    assert direct == table
    assert int(_counters(ctr)["flags"]) == 0


def test_split_launches_and_setup_chunks_agree(ctx):
    """n-range split over launches and power table split over threads give the same bits."""
    g = _golden("config1")
    base = ctx.sieve(g["pmin"], g["pmax"], g["nmin"], g["nmax"])
    try:
        ctx.set_tuning(max_steps_per_launch=137, setup_chunks=5)
        r = ctx.sieve(g["pmin"], g["pmax"], g["nmin"], g["nmax"])
    finally:
        ctx.set_tuning()
    assert (r.raw_sum, r.primecount, r.checksum, r.lines()) == (base.raw_sum, base.primecount, base.checksum,
                                                               base.lines())
    assert f"{r.checksum:016X}" == g["checksum"]


def test_small_segments_agree(ctx):
    """Any segmentation of the p-range gives the same result (sums commute)."""
    g = _golden("selftest3")
    r = ctx.sieve(g["pmin"], g["pmax"], g["nmin"], g["nmax"], seg_width=7_777, threads=8)
    assert f"{r.checksum:016X}" == g["checksum"]
    assert r.primecount == g["primecount"]


def test_hit_overflow_is_reported(ctx):
    """A factor buffer that is too small yields FS_E_OVERFLOW, not silent loss."""
    import factsieve_gb300 as fs
    g = _golden("wilson_small")
    ctx.begin(g["pmin"], g["pmax"], g["nmin"], g["nmax"], result_cap=10)
    ctx.run_range(g["pmin"], g["pmax"])
    hits, raw, pc, flags, rc = ctx.collect(10, raise_on_flags=False)
    assert rc == fs.FS_E_OVERFLOW
    assert flags & fs.FLAG_HIT_OVERFLOW


@pytest.mark.parametrize("lo,hi,nmin,nmax", [
    (10**15, 10**15 + 300_000, 100_000, 100_700),                  # half-offset 96-bit step (p < 2^63, p k > 2^62)
    (10**13, 10**13 + 30_000, 67_109_000, 67_109_700),             # lazy 96-bit step (k_max >= 2^26)
    (10**13, 10**13 + 30_000, 67_108_000, 67_108_800),             # half-offset 96-bit step, k_max just below 2^26
    ((1 << 63) + 1, (1 << 63) + 300_000, 5_000, 5_700),             # half-offset canonical 96-bit step (p >= 2^63)
    ((1 << 63) + 1, (1 << 63) + 10_001, (1 << 26) + 100, (1 << 26) + 700),  # canonical 96-bit step (k_max >= 2^26)
    ((1 << 64) - 20_000, (1 << 64) - 1, (1 << 26) - 800, (1 << 26) - 1),    # half-offset at p near 2^64, k_max near 2^26
    ((1 << 64) - 400_000, (1 << 64) - 1, 1_000, 1_333),              # canonical 96-bit step near 2^64
    (4 * 10**12, 4 * 10**12 + 200_000, 1_000_000, 1_000_300),      # across the 64/96-bit boundary
    (10**12, 10**12 + 300_000, 100_000, 100_700),                  # lazy 64-bit step
    ((1 << 36) + 1, (1 << 36) + 300_000, 500_000, 500_300),        # lazy 64-bit step, large multipliers
    ((1 << 33) - 150_000, (1 << 33) + 150_000, 2000, 2900),         # generic / lazy boundary at 2^33
    ((1 << 31) - 150_000, (1 << 31) + 150_000, 2000, 2900),         # 32-bit / shifted-window boundary at 2^31
    ((1 << 34) + 1, (1 << 34) + 300_001, 20_000, 20_900),          # shifted-window 64-bit step
    ((1 << 32) + 1, (1 << 32) + 20_001, (1 << 25) - 700, (1 << 25) - 1),  # shifted window, k_max just below 2^25
    (10**9, 10**9 + 20_000, 67_108_000, 67_108_800),               # 32-bit step, k_max just below 2^26
    (8 * 10**12, 8 * 10**12 + 300_000, 524_000, 524_400),          # multipliers across 2^19
    ((1 << 36) - 150_000, (1 << 36) + 150_000, 2000, 2900),         # lazy / half-offset boundary at p = 2^36
    ((1 << 40) - 150_000, (1 << 40) + 150_000, 1_047_700, 1 << 20),    # p kmax = 2^60
    ((1 << 40) - 50_000, (1 << 40) + 50_000, 4_193_800, 1 << 22),      # half-offset 64-bit limit p kmax = 2^62
    ((1 << 38) + 1, (1 << 38) + 300_001, 2000, 2900),               # float-quotient step at its floor p = 2^38
    (10**12, 10**12 + 300_000, 441_000, 441_505),                  # float-quotient step at 19 k_max = 2^23
    ((1 << 40) - 150_000, (1 << 40) + 150_000, 400_000, 400_700),  # float-quotient, threads on both sides of 2^40
    ((1 << 50) - 200_000, 1 << 50, 3_500, 4096),                    # float-quotient step at p k_max = 2^62
    ((1 << 56) - 200_000, (1 << 56) - 1, 40, 64),                   # float-quotient step, shift s - 32 = 20
])
def test_walk_regimes_match_oracle(ctx, orc, lo, hi, nmin, nmax):
    """Every walk regime (and a pair straddling two) gives the oracle's residues, sums and hits."""
    import factsieve_gb300 as fs
    want_c = orc.candidates(lo, hi)
    cap = fs.candidate_capacity(lo, hi)
    cand, res, hits, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), nmin, res.data_ptr())
    ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmin, nmax, hits.data_ptr(), 1 << 16)
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmax)
    ctx.synchronize()
    c = _counters(ctr)
    n = int(c["ncand"])
    got_c = _u64(cand)[:n]
    order = np.argsort(got_c)
    assert got_c[order].tolist() == want_c.tolist()
    want = orc.sieve_list(want_c, nmin, nmax, want_residues=True)
    assert _u64(res)[:n][order].tolist() == want["s6"].tolist()
    assert int(c["raw_sum"]) == want["raw_sum"]
    assert int(c["flags"]) == 0
    assert _sorted_hits(_hits_array(hits, int(c["nhits"]))) == _sorted_hits(want["hits"])


def test_walk_with_multipliers_beyond_2p28(ctx, orc):
    """n above 2^28 takes the generic Montgomery walk; still bit-exact."""
    import factsieve_gb300 as fs
    nmin, nmax = (1 << 28) + 5, (1 << 28) + 200
    lo, hi = 10**12, 10**12 + 400
    want_c = orc.candidates(lo, hi)
    assert len(want_c) >= 4
    cap = fs.candidate_capacity(lo, hi)
    cand, res, hits, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), nmin, res.data_ptr())
    ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmin, nmax, hits.data_ptr(), 1 << 16)
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmax)
    ctx.synchronize()
    c = _counters(ctr)
    want = orc.sieve_list(want_c, nmin, nmax)
    assert int(c["raw_sum"]) == want["raw_sum"]
    assert int(c["flags"]) == 0


@pytest.mark.parametrize("name", ["config3_slice100", "config2_slice100", "selftest1", "config3", "config2"])
def test_search_matches_long_fixture(ctx, name):
    g = _golden(name)
    r = ctx.sieve(g["pmin"], g["pmax"], g["nmin"], g["nmax"], threads=16)
    assert (r.primecount, f"{r.raw_sum:016X}", f"{r.checksum:016X}", r.factorcount) == \
        (g["primecount"], g["raw_sum"], g["checksum"], g["factorcount"])


@pytest.mark.parametrize("variant", [3, 5])
@pytest.mark.parametrize("case", [2, 4, 5])
def test_four_candidate_kernel_reference_selftests(ctx, variant, case):
    """The four-candidates-per-thread sieve (two interleaved pairs) on the reference's
    self tests: lazy 64-bit walk (case 2) and lazy 96-bit walk (cases 4, 5), each
    with true factors, so the pair-wise hit replay runs."""
    pmin, pmax, nmin, nmax, fc, pc, cs = SELFTEST[case]
    try:
        ctx.set_tuning(sieve_variant=variant)
        r = ctx.sieve(pmin, pmax, nmin, nmax, threads=16)
    finally:
        ctx.set_tuning()
    assert (r.factorcount, r.primecount, r.checksum) == (fc, pc, cs)


@pytest.mark.parametrize("variant", [3, 5])
@pytest.mark.parametrize("lo,hi,nmin,nmax", [
    ((1 << 63) + 1, (1 << 63) + 300_001, 5_000, 5_700),             # canonical 96-bit walk
    ((1 << 64) - 400_000, (1 << 64) - 1, 1_000, 1_333),              # canonical 96-bit walk near 2^64
    (4 * 10**12, 4 * 10**12 + 200_000, 1_000_000, 1_000_300),      # mixed steps: pairs one after the other
    (10**15 + 1, 10**15 + 300_001, 100_000, 100_701),               # half-offset 96-bit walk
    (10**12 + 7, 10**12 + 300_007, 100_000, 100_701),               # lazy 64-bit, odd n-range (tail steps)
    ((1 << 33) - 150_000, (1 << 33) + 150_000, 2000, 2900),         # generic / lazy boundary
    ((1 << 63) + (1 << 30) - 300_001, (1 << 63) + (1 << 30) - 1, 100_000, 100_301),  # folded setup, d near 2^30
    ((1 << 63) + (1 << 30) - 150_000, (1 << 63) + (1 << 30) + 150_000, 20_000, 20_301),  # folded / Montgomery mix
    ((1 << 63) + 1, (1 << 63) + 50_001, 1_000_000, 1_000_100),      # folded setup of 1e6! (35,800 products)
])
def test_four_candidate_kernel_matches_oracle(ctx, orc, variant, lo, hi, nmin, nmax):
    want = orc.run(lo, hi, nmin, nmax)
    try:
        ctx.set_tuning(sieve_variant=variant)
        r = ctx.sieve(lo, hi, nmin, nmax, seg_width=77_777)       # many segments: ragged candidate counts
    finally:
        ctx.set_tuning()
    assert (r.primecount, r.raw_sum, r.checksum, r.factorcount) == \
        (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"])
    assert r.lines() == [f"{int(p)} | {abs(int(nc))}!{'+1' if nc > 0 else '-1'}"
                         for p, nc in zip(want["factors"]["p"], want["factors"]["nc"])]


# Prime factors p >= 2^31 of n! + c for small n (found by factoring n! +- 1;
# each is re-checked below with an exact factorial): real hits for the
# lazy walks, including the half-offset forms.
KNOWN_FACTORS = [(87178291199, 14, -1), (256443711677, 17, -1), (1713311273363831, 19, 1),
                 (117876683047, 20, 1), (19499250680671, 20, -1), (2703875815783, 21, 1),
                 (4826713612027, 21, -1), (93799610095769647, 22, 1), (170006681813, 22, -1),
                 (148139754736864591, 23, 1), (498390560021687969, 23, -1), (625793187653, 24, -1),
                 (991459181683, 24, -1), (1042190196053, 28, -1), (2778942057555023489, 29, 1),
                 (594278556271609021, 29, -1),
                 # 2^31 <= p < 2^36 (shifted-window step) and p >= 2^63 (96-bit half-offset step)
                 (3790360487, 14, 1), (6880233439, 16, -1), (7798078091, 28, -1),
                 (10398560889846739639, 34, -1)]


@pytest.mark.parametrize("variant", [3, 5])
@pytest.mark.parametrize("p,n,c", KNOWN_FACTORS)
def test_known_large_factors_are_found(ctx, orc, variant, p, n, c):
    import math
    assert (math.factorial(n) + c) % p == 0
    lo, hi, nmin, nmax = p - 3000, p + 3001, 10, 61
    want = orc.exact_small(lo, hi, nmin, nmax)
    assert (p, -n if c < 0 else n) in want["factors"]
    try:
        ctx.set_tuning(sieve_variant=variant)
        r = ctx.sieve(lo, hi, nmin, nmax)
    finally:
        ctx.set_tuning()
    assert (r.primecount, r.raw_sum, r.checksum) == (want["primecount"], want["raw_sum"], want["checksum"])
    assert [(int(q), int(nc)) for q, nc in zip(r.factors["p"], r.factors["nc"])] == want["factors"]


def _random_cases(n, seed, plo=1 << 7, wmax=6000):
    import math
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        lo = int(math.exp(rng.uniform(math.log(plo), math.log((1 << 64) - 2_000_000))))
        width = rng.randrange(20_000, 120_000)
        nmin = int(math.exp(rng.uniform(math.log(34), math.log(300_000))))
        out.append((max(lo, nmin), max(lo, nmin) + width, nmin, nmin + rng.randrange(1, wmax)))
    return out


@pytest.mark.parametrize("lo,hi,nmin,nmax", _random_cases(64, 20261204) + _random_cases(64, 7, 1 << 31, 20_000))
def test_random_ranges_match_oracle(ctx, orc, lo, hi, nmin, nmax):
    """Seeded random p-ranges (log-uniform over [2^7, 2^64)) and n-ranges (nmin
    log-uniform over [34, 3e5)): the whole search (launch-wide step, four
    candidates per thread) and the stage-level path (a step chosen per
    candidate, two per thread) both equal the oracle bit for bit."""
    import factsieve_gb300 as fs
    want = orc.run(lo, hi, nmin, nmax)
    assert want["status"] == 0
    r = ctx.sieve(lo, hi, nmin, nmax)
    assert (r.primecount, r.raw_sum, r.checksum, r.factorcount) == \
        (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"])
    cap = fs.candidate_capacity(lo, hi)
    cand, res, hits, ctr = _dev_buffers(cap)
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), nmin, res.data_ptr())
    ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmin, nmax, hits.data_ptr(), 1 << 16)
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmax)
    ctx.synchronize()
    cs = _counters(ctr)
    assert (int(cs["raw_sum"]), int(cs["flags"]), int(cs["nhits"])) == (want["raw_sum"], 0, want["nhits"])


def _regime_cases(seed):
    """Seeded ranges inside the two forms that need launch-wide proofs: the
    float-quotient walk (p >= 2^38, k_max <= 441,505 and its z bound) and the
    folded setup (p in (2^63, 2^63 + 2^30)), with bounds chosen near their
    edges as often as inside."""
    import random
    import factsieve_gb300 as fs
    rng = random.Random(seed)
    out = []
    while len(out) < 48:
        bits = rng.randrange(38, 60)
        lo = rng.randrange(1 << bits, 1 << (bits + 1))
        kmax = rng.choice([rng.randrange(300, 441_506), rng.randrange(430_000, 441_506)])
        lo, w = rng.choice([(lo, rng.randrange(2000, 40_000)), ((1 << bits) - 20_000, 40_000)])
        nmin = max(34, kmax - rng.randrange(1, 1500))
        if fs.walk_step(lo, lo + w, kmax) == 9:
            out.append((lo, lo + w, nmin, kmax))
    while len(out) < 80:
        d = rng.choice([rng.randrange(0, (1 << 30) - 50_000), (1 << 30) - 40_001])
        lo, w = (1 << 63) + d, rng.randrange(2000, 40_000)
        nmin = rng.choice([rng.randrange(34, 2000), rng.randrange(2000, 300_000)])
        if fs.setup_form(lo, lo + w):
            out.append((lo, lo + w, nmin, nmin + rng.randrange(1, 800)))
    return out


@pytest.mark.parametrize("variant", [5, 3])
def test_random_float_quotient_and_folded_setup_ranges(ctx, orc, variant):
    """Seeded random ranges of the float-quotient walk step and of the folded
    setup products, searched with ragged segment widths by both kernel builds:
    every one equals the oracle bit for bit."""
    import random
    rng = random.Random(5 + variant)
    bad = []
    try:
        ctx.set_tuning(sieve_variant=variant)
        for lo, hi, nmin, nmax in _regime_cases(20261204):
            want = orc.run(lo, hi, nmin, nmax)
            r = ctx.sieve(lo, hi, nmin, nmax, seg_width=rng.choice([7_777, 50_000, 10**6]))
            if (r.primecount, r.raw_sum, r.checksum, r.factorcount) != \
                    (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"]):
                bad.append((lo, hi, nmin, nmax))
    finally:
        ctx.set_tuning()
    assert not bad, bad
