"""The nmax round trip (check.cl:67-78) on the GPU: it fires when the walk did
not cover [nmin, nmax) exactly once.

The reference carries s7 = n * 2^64 mod p in each candidate's record and adds
2^64 once per iterate step (iterate.cl:67-68), so a skipped or repeated
iterate range leaves s7 away from nmax * 2^64 and check.cl flags it
(g_primecount[5]).  Here each residue carries the n it stands at between
stage calls, counted by the walk itself; fs_check derives s7 from it.  The
failures are made on the host (an iterate range left out, or walked twice):
no GPU fault is involved.  Comparisons are exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LO, HI, NMIN, NMAX = 2_000_003, 2_060_000, 3000, 4500


def _counters(ctr):
    import factsieve_gb300 as fs
    return np.frombuffer(ctr.cpu().numpy().tobytes(), dtype=fs.COUNTERS_DTYPE)[0]


def _stage(ctx, chunks, nmax=NMAX):
    """getsegprimes, setup at NMIN, one fs_iterate per (nstart, nend) chunk, fs_check at nmax."""
    import torch
    import factsieve_gb300 as fs
    cap = fs.candidate_capacity(LO, HI)
    cand = torch.zeros(cap, dtype=torch.int64, device="cuda")
    res = torch.zeros(fs.walk_state_words(cap), dtype=torch.int64, device="cuda")
    hits = torch.zeros(2 << 16, dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()   # the library's stream does not wait for torch's fills
    ctx.getsegprimes(LO, HI, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), NMIN, res.data_ptr())
    for s, e in chunks:
        ctx.iterate(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), s, e, hits.data_ptr(), 1 << 16)
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), nmax)
    ctx.synchronize()
    return _counters(ctr)


def test_complete_walk_in_chunks_passes(ctx, orc):
    c = _stage(ctx, [(NMIN, 3100), (3100, 3999), (3999, NMAX)])
    want = orc.sieve_list(orc.candidates(LO, HI), NMIN, NMAX)
    assert want["nvalidfail"] == 0
    assert int(c["flags"]) == 0
    assert int(c["raw_sum"]) == want["raw_sum"]


def test_skipped_iterate_range_fails_the_round_trip(ctx, orc):
    """Walk [NMIN, 3700), skip [3700, NMAX), check at NMAX: every candidate
    fails, and the sum is the reference's for a walk that stopped at 3700
    (s7 = 3700 * 2^64, not NMAX * 2^64)."""
    import factsieve_gb300 as fs
    c = _stage(ctx, [(NMIN, 3700)])
    assert int(c["flags"]) & fs.FLAG_VALIDATION
    want = orc.sieve_list(orc.candidates(LO, HI), NMIN, 3700)
    assert int(c["raw_sum"]) == want["raw_sum"]


def test_repeated_iterate_range_fails_the_round_trip(ctx):
    """[3500, 3700) walked twice: the residues stand 200 steps past NMAX."""
    import factsieve_gb300 as fs
    c = _stage(ctx, [(NMIN, 3700), (3500, NMAX)])
    assert int(c["flags"]) & fs.FLAG_VALIDATION


def test_check_at_the_wrong_nmax_fails(ctx):
    """A complete walk to NMAX checked against NMAX + 1."""
    import factsieve_gb300 as fs
    c = _stage(ctx, [(NMIN, NMAX)], nmax=NMAX + 1)
    assert int(c["flags"]) & fs.FLAG_VALIDATION


@pytest.mark.parametrize("steps", [1, 7, 8, 9, 333])
def test_split_searches_pass_the_round_trip(ctx, orc, steps):
    """A whole search split into launches of a few steps (residues and their n
    carried between launches) raises no flag and equals the oracle."""
    lo, hi, nmin, nmax = 1_000_000, 1_050_000, 1000, 1400
    want = orc.run(lo, hi, nmin, nmax)
    ctx.set_tuning(max_steps_per_launch=steps)
    try:
        r = ctx.sieve(lo, hi, nmin, nmax)
    finally:
        ctx.set_tuning()
    assert (r.primecount, r.raw_sum, r.checksum) == (want["primecount"], want["raw_sum"], want["checksum"])


# one range per walk step (the regimes of tests/test_gpu_parity.py), each searched
# with the n-range cut into short launches: every launch after the first starts
# from stored residues and walked-n tags, and may take a different step as the
# multipliers grow
SPLIT_REGIMES = [
    (10**15, 10**15 + 200_000, 100_000, 100_700),                  # float quotient, 96-bit product
    (10**15, 10**15 + 200_000, 1_276_000, 1_277_000),              # ... into the half-offset 96-bit step at its k_max bound
    (10**13, 10**13 + 30_000, 67_108_000, 67_109_700),             # half-offset 96-bit into lazy 96-bit at 2^26
    ((1 << 63) + 1, (1 << 63) + 200_000, 5_000, 5_700),             # half-offset canonical 96-bit, float quotient
    ((1 << 63) + 1, (1 << 63) + 20_001, 1_276_000, 1_277_000),      # ... into the integer quotient at its k_max bound
    ((1 << 63) + 1, (1 << 63) + 10_001, (1 << 26) - 300, (1 << 26) + 400),  # into canonical 96-bit at 2^26
    ((1 << 64) - 200_000, (1 << 64) - 1, 1_000, 1_333),              # near 2^64
    (10**12, 10**12 + 200_000, 100_000, 100_700),                  # float quotient, window from the least p
    (10**12, 10**12 + 200_000, 441_000, 442_000),                  # ... into the k_max-aware window
    (10**12, 10**12 + 200_000, 1_276_000, 1_277_000),              # ... into the half-offset lazy 64-bit step
    ((1 << 34) + 1, (1 << 34) + 200_001, 20_000, 20_900),          # float quotient, window shift <= 32
    ((1 << 34) + 1, (1 << 34) + 200_001, 1_276_000, 1_277_000),    # ... into the shifted-window step
    ((1 << 31) - 100_000, (1 << 31) + 100_000, 2000, 2900),         # across 2^31: a step per candidate
    (10**9, 10**9 + 20_000, 67_108_000, 67_109_000),               # 32-bit step into the generic walk
    ((1 << 33) - 100_000, (1 << 33) + 100_000, 2000, 2900),         # float quotient across 2^33
    (1_000_000, 1_100_000, 1000, 3000),                            # small p, many hits
]


@pytest.mark.parametrize("lo,hi,nmin,nmax", SPLIT_REGIMES)
@pytest.mark.parametrize("steps", [97, 1000])
def test_split_walks_in_every_regime_equal_the_oracle(ctx, orc, lo, hi, nmin, nmax, steps):
    want = orc.run(lo, hi, nmin, nmax)
    assert want["status"] == 0
    ctx.set_tuning(max_steps_per_launch=steps)
    try:
        r = ctx.sieve(lo, hi, nmin, nmax)
    finally:
        ctx.set_tuning()
    assert (r.primecount, r.raw_sum, r.checksum, r.factorcount) == \
        (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"])
