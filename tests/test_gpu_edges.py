"""Edge cases and failure paths on the GPU, through the C ABI.

Empty p- and n-ranges, a candidate buffer too small for its segment (the
true count is still reported and the overflow is flagged, never silently
truncated), and the plan check for a caller-supplied setup plan: a correct
plan multiplies to nmin! mod p, a corrupted one raises FS_FLAG_TABLE.
All comparisons are exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _counters(ctr):
    import factsieve_gb300 as fs
    return np.frombuffer(ctr.cpu().numpy().tobytes(), dtype=fs.COUNTERS_DTYPE)[0]


def _plan_on_device(fs, nmin):
    import torch
    words, layers, deficit = fs.setup_plan(nmin)
    words = np.concatenate([words, np.zeros(1, np.uint64)])   # d_words is non-null even when 2! needs no word
    dw = torch.from_numpy(words.view(np.int64).copy()).cuda()
    dl = torch.from_numpy(layers.astype(np.uint32).reshape(-1).view(np.int32).copy()).cuda()
    torch.cuda.synchronize()
    return dw, dl, len(layers), deficit


def _candidates(ctx, lo, hi):
    import torch
    import factsieve_gb300 as fs
    cap = fs.candidate_capacity(lo, hi)
    cand = torch.zeros(cap, dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()   # the library's stream does not wait for torch's fills
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    return cand, ctr


def test_empty_p_range(ctx):
    r = ctx.sieve(10**12, 10**12, 1000, 2000)
    assert (r.primecount, r.factorcount, r.checksum, len(r.factors)) == (0, 0, 0, 0)
    # a range holding no candidate: 1e12+1..1e12+9 has no number free of factors <= 113 that is a 2-PRP
    r = ctx.sieve(10**12 + 1, 10**12 + 10, 1000, 2000)
    assert r.primecount == 0 and r.checksum == 0


@pytest.mark.parametrize("lo,hi,n", [(1_000_000, 1_100_000, 1000), (10**12, 10**12 + 200_000, 100_000)])
def test_empty_n_range_matches_oracle(ctx, orc, lo, hi, n):
    """nmin == nmax walks no step; the checksum is still sum(nmin! R + nmax R) over the candidates."""
    want = orc.run(lo, hi, n, n)
    r = ctx.sieve(lo, hi, n, n)
    assert (r.primecount, r.checksum, r.factorcount) == (want["primecount"], want["checksum"], 0)


@pytest.mark.parametrize("nmin", [1, 2, 3, 4, 5, 6, 20, 33])
def test_smallest_nmin_is_exact(ctx, orc, nmin):
    """Below nmin = 34 the reference's setup (nmin < 4) or verifier (hits with
    n < 34) is wrong, so the definition itself is the oracle here."""
    want = orc.exact_small(127, 60_000, nmin, 400)
    r = ctx.sieve(127, 60_000, nmin, 400)
    assert (r.primecount, r.raw_sum, r.checksum, r.factorcount) == \
        (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"])
    assert [(int(p), int(nc)) for p, nc in zip(r.factors["p"], r.factors["nc"])] == want["factors"]


def test_candidate_overflow_is_counted_and_flagged(ctx, orc):
    import torch
    import factsieve_gb300 as fs
    lo, hi, cap = 1_000_000, 1_200_000, 10
    cand = torch.zeros(cap, dtype=torch.int64, device="cuda")
    res = torch.zeros(fs.walk_state_words(cap), dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    ctx.getsegprimes(lo, hi, cand.data_ptr(), cap, ctr.data_ptr())
    want = orc.candidates(lo, hi)
    c = _counters(ctr)
    assert int(c["ncand"]) == len(want) > cap         # the true count, not the capacity
    got = set(cand.cpu().numpy().view(np.uint64).tolist())
    assert got <= set(int(x) for x in want)           # the slots that fit hold real candidates
    ctx.setup(cand.data_ptr(), cap, ctr.data_ptr(), 1000, res.data_ptr())
    ctx.check(cand.data_ptr(), cap, ctr.data_ptr(), res.data_ptr(), 1000)
    assert int(_counters(ctr)["flags"]) & fs.FLAG_CAND_OVERFLOW


@pytest.mark.parametrize("nmin", [2, 127, 100_000, 3_000_000])
def test_plan_check_accepts_the_library_plan(ctx, nmin):
    import factsieve_gb300 as fs
    cand, ctr = _candidates(ctx, 1_000_000_000_039, 1_000_000_100_000)
    dw, dl, nl, deficit = _plan_on_device(fs, nmin)
    direct, table = ctx.plan_check(cand.data_ptr(), ctr.data_ptr(), nmin, dw.data_ptr(), dl.data_ptr(), nl, deficit)
    assert direct == table
    assert int(_counters(ctr)["flags"]) == 0
    # the same value the library's own plan gives
    assert ctx.table_check(cand.data_ptr(), ctr.data_ptr(), nmin) == (direct, table)


@pytest.mark.parametrize("what", ["word", "deficit", "nmin"])
def test_plan_check_flags_a_corrupted_plan(ctx, what):
    import factsieve_gb300 as fs
    nmin = 100_000
    cand, ctr = _candidates(ctx, 1_000_000_000_039, 1_000_000_100_000)
    dw, dl, nl, deficit = _plan_on_device(fs, nmin)
    n_check = nmin
    if what == "word":
        dw[(len(dw) - 1) // 2] += 2      # one packed word of the product changed
    elif what == "deficit":
        deficit += 1
    else:
        n_check = nmin + 1               # the plan of nmin checked against (nmin+1)!
    direct, table = ctx.plan_check(cand.data_ptr(), ctr.data_ptr(), n_check, dw.data_ptr(), dl.data_ptr(), nl,
                                   deficit)
    assert direct != table
    assert int(_counters(ctr)["flags"]) & fs.FLAG_TABLE


def test_ceiling_kernels_report_rates(ctx):
    """The roofline's ceiling microkernels (fs_bench_int_pipe kinds 0-19) run and
    report plausible rates; an unknown kind is refused, and so are iterations
    that would take the k_max-window float-quotient kinds (16-19) past their
    multiplier bound."""
    import factsieve_gb300 as fs
    rates = {k: ctx.bench_int_pipe(k, 200)[0] for k in range(20)}
    assert all(v > 0 for v in rates.values()), rates
    assert rates[0] > rates[4]             # an IMAD issues faster than a Montgomery product completes
    with pytest.raises(fs.FSError):
        ctx.bench_int_pipe(20, 200)
    with pytest.raises(fs.FSError):
        ctx.bench_int_pipe(5, 0)
    ctx.bench_int_pipe(17, 147_065)        # multipliers up to 100,001 + 8 x 147,065 = 1,276,521
    with pytest.raises(fs.FSError):
        ctx.bench_int_pipe(17, 147_066)


def test_pending_count_sizes_collect(ctx, orc):
    """fs_search_pending reports, without clearing, the records the next collect
    returns; collect then copies exactly those."""
    import numpy as np
    import factsieve_gb300 as fs
    lo, hi, nmin, nmax = 127, 100_000, 127, 2_000
    want = orc.run(lo, hi, nmin, nmax)
    ctx.begin(lo, hi, nmin, nmax)
    ctx.segment(lo, hi)
    pend = np.zeros(1, np.uint64)
    assert fs.lib().fs_search_pending(ctx.handle, fs._p64(pend)) == 0
    assert int(pend[0]) == want["nhits"] > 0
    assert fs.lib().fs_search_pending(ctx.handle, fs._p64(pend)) == 0      # unchanged: nothing cleared
    assert int(pend[0]) == want["nhits"]
    hits, raw, pc, flags, rc = ctx.collect(1 << 20)
    assert (len(hits), raw, pc, rc) == (want["nhits"], want["raw_sum"], want["primecount"], 0)
    assert fs.lib().fs_search_pending(ctx.handle, fs._p64(pend)) == 0
    assert int(pend[0]) == 0                                                # collect cleared them


@pytest.mark.parametrize("nmin", [127, 5000])
def test_table_check_without_candidates_uses_a_fixed_prime(ctx, nmin):
    """A segment with no candidate still checks the power table, against 2^61 - 1."""
    import math
    import torch
    cand = torch.zeros(1, dtype=torch.int64, device="cuda")
    ctr = torch.zeros(4, dtype=torch.int64, device="cuda")          # ncand = 0
    torch.cuda.synchronize()
    direct, table = ctx.table_check(cand.data_ptr(), ctr.data_ptr(), nmin)
    q = (1 << 61) - 1
    assert direct == table == math.factorial(nmin) * (1 << 64) % q
    assert int(_counters(ctr)["flags"]) == 0
