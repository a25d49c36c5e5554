"""The batched persistent form: every job's result in a mixed batch equals the
same job searched alone (bit for bit), across all walk regimes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# deliberately uneven jobs: small p (generic walk), lazy 64-bit, lazy 96-bit,
# canonical 96-bit (p >= 2^63), a large nmin (long setup), many hits, nmin = nmax
JOBS = [
    (1_000_000, 1_300_000, 1000, 2500),
    (127, 20_000, 127, 30_000),
    (10**12, 10**12 + 3_000_000, 100_000, 101_500),
    (10**15, 10**15 + 2_000_000, 200_000, 200_900),
    ((1 << 63) + 11, (1 << 63) + 2_000_000, 1_000_000, 1_000_700),
    (5 * 10**11, 5 * 10**11 + 500_000, 2_000_000, 2_000_100),
    ((1 << 62) - 1_000_000, (1 << 62) + 1_000_000, 3000, 3600),
    (10**9, 10**9 + 1_000_000, 5000, 5000),
]


def _hits(r):
    return sorted(zip(r.factors["p"].tolist(), r.factors["nc"].tolist()))


def test_batch_equals_each_job_alone(ctx):
    alone = [ctx.sieve(*j, threads=8) for j in JOBS]
    batch = ctx.batch_sieve(JOBS, threads=8)
    assert len(batch) == len(JOBS)
    for j, a, b in zip(JOBS, alone, batch):
        assert (b.primecount, b.raw_sum, b.checksum, b.factorcount, b.nhits) == \
            (a.primecount, a.raw_sum, a.checksum, a.factorcount, a.nhits), j
        assert _hits(b) == _hits(a), j


def test_batch_graph_replays_identically(ctx):
    jobs = JOBS[:4]
    ctx.batch_prepare(jobs)
    outs = []
    for _ in range(3):
        ctx.batch_launch()
        res, hits, rc = ctx.batch_collect()
        assert rc == 0
        outs.append((res, sorted(zip(hits["p"].tolist(), hits["nc"].tolist(), hits["pad"].tolist()))))
    assert outs[0] == outs[1] == outs[2]
    ctx.batch_release()


def test_batch_matches_oracle(ctx, orc):
    jobs = [JOBS[0], JOBS[1], JOBS[7]]
    got = ctx.batch_sieve(jobs, threads=8)
    for j, g in zip(jobs, got):
        w = orc.run(*j)
        assert (g.primecount, g.checksum, g.factorcount) == (w["primecount"], w["checksum"], w["factorcount"]), j


def _config4_slices():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "run_config4_slices.json")
    with open(path) as fh:
        return json.load(fh)["jobs"]


def test_config4_mix_on_slices_matches_oracle(ctx):
    """The 64-job mix (seed 1) with each p-range cut to its first 1/1000, as
    one batch: every job equals the oracle's search of it (the fixture
    run_config4_slices.json, made by tests/golden/make_golden.py)."""
    want = _config4_slices()
    jobs = [(j["pmin"], j["pmax"], j["nmin"], j["nmax"]) for j in want]
    got = ctx.batch_sieve(jobs, threads=8)
    for j, g, w in zip(jobs, got, want):
        assert (g.primecount, g.raw_sum, g.checksum, g.factorcount, g.nhits) == \
            (w["primecount"], int(w["raw_sum"], 16), int(w["checksum"], 16), w["factorcount"], w["nhits"]), j


def test_config4_mix_on_slices_served_matches_oracle(ctx):
    """The same 64 sliced jobs through the serving loop, submitted in the
    stream's order while earlier ones are resident."""
    import factsieve_gb300 as fs
    from factsieve_gb300.serve import Server
    want = _config4_slices()
    srv = Server(ctx, max_active=16, round_budget=3_000_000_000, mem_reserve=1 << 30)
    done = {}
    try:
        for k, j in enumerate(want):
            srv.submit((j["pmin"], j["pmax"], j["nmin"], j["nmax"]), k)
            if k % 4 == 3:
                srv.round()
                for d in srv.poll():
                    done[d["id"]] = d
        rounds = 0
        while len(done) < len(want):
            srv.round()
            rounds += 1
            for d in srv.poll():
                done[d["id"]] = d
            assert rounds < 20000
    finally:
        srv.close()
    for k, w in enumerate(want):
        d = done[k]
        kept, cs_add, _ = fs.postprocess(d["hits"], threads=8)
        assert d["flags"] == 0
        assert (d["primecount"], d["raw_sum"], (d["raw_sum"] + cs_add) & ((1 << 64) - 1)) == \
            (w["primecount"], int(w["raw_sum"], 16), int(w["checksum"], 16)), k
