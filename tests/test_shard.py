"""Multi-rank path: world-size-2 gloo groups shard one search over p, each
rank computes its shard (with the oracle on CPU, or on the GPU under -m gpu),
and the host combine equals the single-rank search bit for bit.  A failing
rank surfaces as an error on the other rank, not a hang."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_compute(nmin, nmax):
    def run(lo, hi):
        import oracle
        import factsieve_gb300 as fs
        r = oracle.run(lo, hi, nmin, nmax)
        assert r["status"] == 0
        return fs.SieveResult(r["factors"], r["checksum"], r["primecount"], r["factorcount"], r["raw_sum"],
                              r["nhits"], r["ndiscarded"])
    return run


def _worker(rank, world, port, job, fail_rank, out, gpu=False):
    import sys
    sys.path.insert(0, ROOT)
    import datetime
    import torch.distributed as dist
    from factsieve_gb300.shard import sieve_distributed
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    try:
        pmin, pmax, nmin, nmax = job
        compute = None if gpu else _oracle_compute(nmin, nmax)   # None: this rank's GPU (Context.sieve)
        if rank == fail_rank:
            def compute(lo, hi):
                raise RuntimeError("injected failure on this rank")
        r = sieve_distributed(pmin, pmax, nmin, nmax, compute=compute)
        out[rank] = ("ok", r.primecount, r.checksum, r.factorcount,
                     [(int(p), int(nc)) for p, nc in zip(r.factors["p"], r.factors["nc"])])
    except Exception as e:   # reported to the parent
        out[rank] = ("error", type(e).__name__, str(e)[:200])
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def _run(world, job, fail_rank=-1, gpu=False):
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, job, fail_rank, out, gpu)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        if p.is_alive():
            p.kill()
    return dict(out)


def test_two_rank_shards_combine_to_the_whole_search(orc):
    job = (1_000_000, 1_400_000, 1000, 2000)
    whole = orc.run(*job)
    res = _run(2, job)
    assert set(res) == {0, 1}
    for r in res.values():
        assert r[0] == "ok", r
        assert (r[1], r[2], r[3]) == (whole["primecount"], whole["checksum"], whole["factorcount"])
        assert r[4] == [(int(p), int(nc)) for p, nc in zip(whole["factors"]["p"], whole["factors"]["nc"])]


@pytest.mark.gpu
def test_two_rank_gpu_shards_combine_to_the_whole_search(orc):
    """The same with each rank searching its shard on the GPU (sieve_distributed's
    default compute).  This run has one GPU, so both ranks share cuda:0; their
    kernels are independent (nothing on the device waits for the other rank)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    job = (1_000_000_000_000, 1_000_002_000_000, 100_000, 101_000)
    whole = orc.run(*job)
    res = _run(2, job, gpu=True)
    assert set(res) == {0, 1}
    for r in res.values():
        assert r[0] == "ok", r
        assert (r[1], r[2], r[3]) == (whole["primecount"], whole["checksum"], whole["factorcount"])


def test_failed_rank_is_reported_not_hung():
    job = (1_000_000, 1_100_000, 1000, 1200)
    res = _run(2, job, fail_rank=1)
    assert res[1][0] == "error" and "injected failure" in res[1][2]
    assert res[0][0] == "error"          # the healthy rank's gather fails instead of hanging


def test_shard_bounds_and_round_robin_tile_the_range():
    from factsieve_gb300.shard import round_robin_segments, shard_bounds
    for world in (1, 2, 3, 8):
        spans = [shard_bounds(10**12, 10**12 + 999_999_937, world, r) for r in range(world)]
        assert spans[0][0] == 10**12 and spans[-1][1] == 10**12 + 999_999_937
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
        segs = sorted(s for r in range(world) for s in round_robin_segments(127, 10**6 + 3, 77_777, world, r))
        assert segs[0][0] == 127 and segs[-1][1] == 10**6 + 3
        assert all(a[1] == b[0] for a, b in zip(segs, segs[1:]))


def test_combine_is_order_independent():
    import factsieve_gb300 as fs
    from factsieve_gb300.shard import combine
    rng = np.random.default_rng(0)
    parts = []
    for _ in range(4):
        f = np.zeros(5, fs.FACTOR_DTYPE)
        f["p"] = rng.integers(10**6, 10**7, 5)
        f["nc"] = rng.integers(-3000, 3000, 5)
        parts.append(fs.SieveResult(f, int(rng.integers(0, 2**63)) * 2, 10, 5, 3, 5, 0))
    a, b = combine(parts), combine(parts[::-1])
    assert (a.checksum, a.primecount, a.factors.tolist()) == (b.checksum, b.primecount, b.factors.tolist())
