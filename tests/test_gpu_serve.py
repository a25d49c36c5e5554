"""The serving loop: jobs admitted while others are resident, advanced in
shared rounds with residues kept on the device, each finish with the same
bits as the job searched alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from test_gpu_batch import JOBS


@pytest.mark.parametrize("budget", [100_000_000, 2_000_000_000, 10**13])
def test_served_jobs_equal_each_job_alone(ctx, budget):
    """A small round budget forces many rounds (setup split over candidates,
    walks split into chunks, jobs joining while others are mid-walk); a large
    one serves each job whole in one chunk; 2e9 mixes both."""
    import factsieve_gb300 as fs
    from factsieve_gb300.serve import Server
    alone = {k: ctx.sieve(*j, threads=8) for k, j in enumerate(JOBS)}
    srv = Server(ctx, max_active=3, round_budget=budget, mem_reserve=1 << 30)
    done = {}
    pending = list(enumerate(JOBS))
    rounds = 0
    try:
        while len(done) < len(JOBS):
            if pending and rounds % 2 == 0:
                k, j = pending.pop(0)
                srv.submit(j, k)
            srv.round()
            rounds += 1
            for d in srv.poll():
                done[d["id"]] = d
            assert rounds < 5000
    finally:
        srv.close()
    assert rounds > len(JOBS) or budget >= 10**13
    for k, d in done.items():
        a = alone[k]
        kept, cs_add, disc = fs.postprocess(d["hits"], threads=8)
        assert d["flags"] == 0, JOBS[k]
        assert (d["primecount"], d["raw_sum"], len(d["hits"])) == (a.primecount, a.raw_sum, a.nhits), JOBS[k]
        assert (d["raw_sum"] + cs_add) & ((1 << 64) - 1) == a.checksum
        assert kept[["p", "nc"]].tolist() == a.factors[["p", "nc"]].tolist()
        assert d["t_submit"] <= d["t_admit"] <= d["t_done"]


def test_admission_waits_for_device_memory(ctx):
    from factsieve_gb300.serve import Server
    srv = Server(ctx, max_active=4, mem_reserve=1 << 60)   # more than any GPU has
    try:
        srv.submit(JOBS[0], 7)
        active, queued = srv.round()
        assert (active, queued) == (0, 1)
        assert srv.poll() == []
    finally:
        srv.close()


def test_large_round_in_four_candidate_form(ctx):
    """Rounds with more tiles than the GPU holds run four candidates per thread,
    small ones two (the other tests): both give each job's bits alone."""
    import factsieve_gb300 as fs
    from factsieve_gb300.serve import Server
    jobs = [(10**12, 10**12 + 10**7, 100_000, 100_300), (2 * 10**12, 2 * 10**12 + 10**7, 50_000, 50_200),
            ((1 << 63) + 1, (1 << 63) + 10**7, 1000, 1200)]
    alone = {k: ctx.sieve(*j, threads=8) for k, j in enumerate(jobs)}
    srv = Server(ctx, max_active=4, round_budget=10**13, mem_reserve=1 << 30)
    done = {}
    try:
        for k, j in enumerate(jobs):
            srv.submit(j, k)
        rounds = 0
        while len(done) < len(jobs):
            srv.round()
            rounds += 1
            for d in srv.poll():
                done[d["id"]] = d
            assert rounds < 100
    finally:
        srv.close()
    for k, d in done.items():
        a = alone[k]
        assert d["flags"] == 0
        assert (d["primecount"], d["raw_sum"], len(d["hits"])) == (a.primecount, a.raw_sum, a.nhits), jobs[k]
