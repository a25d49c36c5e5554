"""Multi-GPU sharding of one search over the p-range.

Candidates are independent, so ranks (one process per GPU) take disjoint
p-ranges and nothing crosses ranks on the data path.  The combine step is on
the host: primecounts add, the checksum adds modulo 2^64 (the reference sums
per-workgroup partial checksums the same way, cl_sieve.cpp:445-449), and the
factor lists concatenate and sort by (p, |n|).

``sieve_distributed`` runs inside a torch.distributed group: each rank
searches its shard (on its own GPU by default) and the results are gathered
as Python objects; with a process-group timeout, a rank that dies or never
joins turns into an error on the others instead of a hang.
"""
from __future__ import annotations

import numpy as np

from . import FACTOR_DTYPE, SieveResult

__all__ = ["shard_bounds", "round_robin_segments", "combine", "sieve_distributed"]


def shard_bounds(pmin: int, pmax: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous share [lo, hi) of [pmin, pmax) for `rank` of `world`; the
    shares tile the range exactly (candidate density is uniform to first
    order over the narrow ranges a search covers)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    span = pmax - pmin
    lo = pmin + span * rank // world
    hi = pmin + span * (rank + 1) // world
    return lo, hi


def round_robin_segments(pmin: int, pmax: int, seg: int, world: int, rank: int):
    """Segments [lo, hi) of width `seg` dealt round-robin to ranks (the dealing
    bench.py uses for weak scaling)."""
    out = []
    lo = pmin
    i = 0
    while lo < pmax:
        hi = min(lo + seg, pmax)
        if i % world == rank:
            out.append((lo, hi))
        lo = hi
        i += 1
    return out


def combine(results) -> SieveResult:
    """Merge per-shard results of one search into the whole search's result."""
    factors = np.concatenate([r.factors for r in results]) if results else np.zeros(0, FACTOR_DTYPE)
    if len(factors):
        key = np.lexsort((np.abs(factors["nc"].astype(np.int64)), factors["p"]))
        factors = factors[key]
    M = (1 << 64) - 1
    return SieveResult(
        factors=factors,
        checksum=sum(int(r.checksum) for r in results) & M,
        primecount=sum(int(r.primecount) for r in results),
        factorcount=sum(int(r.factorcount) for r in results),
        raw_sum=sum(int(r.raw_sum) for r in results) & M,
        nhits=sum(int(r.nhits) for r in results),
        ndiscarded=sum(int(r.ndiscarded) for r in results),
    )


def _gpu_compute(nmin, nmax, threads):
    def run(lo, hi):
        import torch
        from . import Context
        with Context(torch.cuda.current_device()) as ctx:
            return ctx.sieve(lo, hi, nmin, nmax, threads=threads)
    return run


def sieve_distributed(pmin, pmax, nmin, nmax, group=None, compute=None, threads=2):
    """Search [pmin, pmax) x [nmin, nmax) across the ranks of a torch.distributed
    group; every rank returns the combined result.  `compute(lo, hi)` searches
    one shard (default: this rank's GPU through Context.sieve)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_bounds(pmin, pmax, world, rank)
    fn = compute or _gpu_compute(nmin, nmax, threads)
    mine = fn(lo, hi) if hi > lo else SieveResult(np.zeros(0, FACTOR_DTYPE), 0, 0, 0)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine, group=group)
    return combine(gathered)
