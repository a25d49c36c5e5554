"""Segments wider than 2^27 generator words (p-widths beyond 2^33 = 8.6e9).

The candidate generator works on words of 32 consecutive odd numbers, word w
covering o0 + 64 w .. o0 + 64 w + 62.  A generator that indexed survivors by
a 32-bit odd-number offset from o0 would wrap at w = 2^27; these tests run
one launch across that word and compare the candidates there with the
oracle's, and a 1.2e10-wide segment with the same range cut into twelve.
The reference never runs a segment wider than 4,294,900,000
(cl_sieve.cpp:625-627); the C ABI here accepts up to 2^31 words.
All comparisons are exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _counters(ctr):
    import factsieve_gb300 as fs
    return np.frombuffer(ctr.cpu().numpy().tobytes(), dtype=fs.COUNTERS_DTYPE)[0]


def test_candidates_across_generator_word_2p27_match_oracle(ctx, orc):
    """One fs_getsegprimes launch over [1e12, 1e12 + 2^33 + 2e6): the
    candidates in a 2e6-wide window around word 2^27 equal the oracle's."""
    import torch
    import factsieve_gb300 as fs
    low = 10**12
    o0 = low | 1
    edge = o0 + 64 * (1 << 27)                   # first odd number of word 2^27
    high = edge + 2_000_000
    cap = fs.candidate_capacity(low, high)
    cand = torch.zeros(cap, dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()   # the library's stream does not wait for torch's fills
    ctx.getsegprimes(low, high, cand.data_ptr(), cap, ctr.data_ptr())
    ctx.synchronize()
    n = int(_counters(ctr)["ncand"])
    assert n <= cap
    wlo, whi = edge - 1_000_000, edge + 1_000_000
    got = cand[:n]
    got = got[(got >= wlo) & (got < whi)]
    got = np.sort(got.cpu().numpy().view(np.uint64))
    want = orc.candidates(wlo, whi)
    assert len(want) > 10_000
    assert got.tolist() == want.tolist()
    # nothing below low or at/above high, and no number twice
    allc = cand[:n]
    assert int(allc.min()) >= low and int(allc.max()) < high
    assert int(torch.unique(allc).numel()) == n
    del cand, allc, got
    torch.cuda.empty_cache()


def test_wide_segment_equals_twelve_narrow_ones(fslib):
    """fs_search_segment over [1e12, 1e12 + 1.2e10) in one piece gives the
    primecount and raw sum of the same range as twelve 1e9-wide segments.
    (A context of its own: its 8 GB candidate buffer goes with it.)"""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    low, width, nmin, nmax = 10**12, 12 * 10**9, 1000, 1001
    with fslib.Context(0) as c:
        c.begin(low, low + width, nmin, nmax)
        c.segment(low, low + width)
        _, raw1, pc1, fl1, rc1 = c.collect(1 << 20)
        c.begin(low, low + width, nmin, nmax)
        c.run_range(low, low + width, 10**9)
        _, raw12, pc12, fl12, rc12 = c.collect(1 << 20)
    assert (rc1, fl1, rc12, fl12) == (0, 0, 0, 0)
    assert pc1 > 4 * 10**8
    assert (pc1, raw1) == (pc12, raw12)
