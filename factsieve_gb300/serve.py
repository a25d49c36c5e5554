"""Serving loop: continuous batching of sieve requests on one GPU.

``Server`` wraps the library's request loop (fs_serve_* in
include/factsieve.h): requests queue on the host, each round admits jobs
while slots and device memory allow, advances every resident job by an equal
share of the round's work (residues stay on the device between rounds), and
retires the finished ones.  ``run_stream`` replays a timed request stream in
real time and reports offered versus served load and sojourn-time
percentiles (arrival to result).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import FACTOR_DTYPE, Factor, FSError, Job, lib

__all__ = ["Server", "run_stream"]


class Served(C.Structure):
    _fields_ = [("id", C.c_int64), ("raw_sum", C.c_uint64), ("primecount", C.c_uint64), ("nhits", C.c_uint64),
                ("flags", C.c_uint32), ("pad", C.c_uint32), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("hit_offset", C.c_uint64)]


class ServeConfig(C.Structure):
    _fields_ = [("max_active", C.c_uint32), ("hitcap", C.c_uint32), ("round_budget", C.c_uint64),
                ("mem_reserve", C.c_uint64)]


_declared = False


def _declare():
    global _declared
    if _declared:
        return
    L = lib()
    vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    L.fs_clock.restype = C.c_double
    L.fs_clock.argtypes = []
    L.fs_serve_create.restype = C.c_int
    L.fs_serve_create.argtypes = [vp, C.POINTER(ServeConfig)]
    L.fs_serve_submit.restype = C.c_int
    L.fs_serve_submit.argtypes = [vp, C.POINTER(Job), C.c_int64]
    L.fs_serve_round.restype = C.c_int
    L.fs_serve_round.argtypes = [vp, C.POINTER(u32), C.POINTER(u32)]
    L.fs_serve_poll.restype = C.c_int
    L.fs_serve_poll.argtypes = [vp, C.POINTER(Served), u32, C.POINTER(u32), C.POINTER(Factor), u64,
                                C.POINTER(u64)]
    L.fs_serve_stats.restype = C.c_int
    L.fs_serve_stats.argtypes = [vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.fs_serve_destroy.restype = C.c_int
    L.fs_serve_destroy.argtypes = [vp]
    _declared = True


def clock() -> float:
    _declare()
    return lib().fs_clock()


class Server:
    """The request loop of one Context."""

    def __init__(self, ctx, max_active=64, hitcap=1 << 20, round_budget=0, mem_reserve=8 << 30):
        _declare()
        self.ctx = ctx
        cfg = ServeConfig(max_active, hitcap, round_budget, mem_reserve)
        rc = lib().fs_serve_create(ctx.handle, C.byref(cfg))
        if rc:
            raise FSError(rc, "fs_serve_create")
        self.hitcap = hitcap

    def submit(self, job, ident: int) -> None:
        j = Job(*map(int, job))
        rc = lib().fs_serve_submit(self.ctx.handle, C.byref(j), int(ident))
        if rc:
            raise FSError(rc, f"fs_serve_submit({job})")

    def round(self):
        a, q = C.c_uint32(0), C.c_uint32(0)
        rc = lib().fs_serve_round(self.ctx.handle, C.byref(a), C.byref(q))
        if rc:
            raise FSError(rc, "fs_serve_round " + lib().fs_last_error(self.ctx.handle).decode())
        return a.value, q.value

    def poll(self, cap=4096):
        """Finished jobs: list of dicts (id, raw_sum, primecount, flags, times, hits array)."""
        out = (Served * cap)()
        hits = (Factor * self.hitcap)()
        n, nh = C.c_uint32(0), C.c_uint64(0)
        rc = lib().fs_serve_poll(self.ctx.handle, out, cap, C.byref(n), hits, self.hitcap, C.byref(nh))
        if rc:
            raise FSError(rc, "fs_serve_poll")
        harr = np.frombuffer(hits, dtype=FACTOR_DTYPE, count=nh.value).copy()
        res = []
        for k in range(n.value):
            s = out[k]
            d = {f: getattr(s, f) for f, _ in Served._fields_}
            d["hits"] = harr[s.hit_offset:s.hit_offset + s.nhits].copy()
            res.append(d)
        return res

    def stats(self):
        r, s = C.c_uint64(0), C.c_uint64(0)
        su, km = C.c_double(0), C.c_double(0)
        lib().fs_serve_stats(self.ctx.handle, C.byref(r), C.byref(s), C.byref(su), C.byref(km))
        return {"rounds": r.value, "served_pair_steps": s.value, "setup_units": su.value, "kernel_ms": km.value}

    def close(self):
        if self.ctx is not None:
            lib().fs_serve_destroy(self.ctx.handle)
            self.ctx = None


def _pct(xs, q):
    return float(np.percentile(np.array(xs), q)) if xs else None


def run_stream(ctx, requests, stop_after_s, max_active=64, round_budget=0, mem_reserve=8 << 30,
               pair_steps_of=None):
    """Replay `requests` [(arrival_s, pmin, pmax, nmin, nmax), ...] in real time.

    Submits each request at its arrival time, runs rounds while anything is
    resident or queued, and stops when every request is done or `stop_after_s`
    seconds have passed.  Returns (summary dict, {id: finished record})."""
    srv = Server(ctx, max_active=max_active, round_budget=round_budget, mem_reserve=mem_reserve)
    reqs = sorted(enumerate(requests), key=lambda x: x[1][0])
    done = {}
    i = 0
    t0 = clock()
    active = queued = 0
    try:
        fresh = False   # requests submitted since the last round
        while True:
            now = clock() - t0
            while i < len(reqs) and reqs[i][1][0] <= now:
                ident, r = reqs[i]
                srv.submit(r[1:5], ident)
                i += 1
                fresh = True
            if now >= stop_after_s:
                break
            if not fresh and active == 0 and queued == 0:
                if i >= len(reqs):
                    break
                time.sleep(max(0.0, min(reqs[i][1][0] - now, 0.05)))
                continue
            active, queued = srv.round()
            fresh = False
            for d in srv.poll():
                done[d["id"]] = d
        elapsed = clock() - t0
        st = srv.stats()
    finally:
        srv.close()
    submitted = i
    lat = [d["t_done"] - d["t_submit"] for d in done.values()]
    # every submitted request, an unfinished one at its age when the window
    # closed (a lower bound on its sojourn): percentiles that do not drop the
    # requests an overloaded loop could not finish
    ages = [done[ident]["t_done"] - done[ident]["t_submit"] if ident in done else max(elapsed - r[0], 0.0)
            for ident, r in reqs[:submitted]]
    summary = {
        "requests": len(requests), "submitted": submitted, "completed": len(done),
        "unfinished": submitted - len(done), "elapsed_s": elapsed, "rounds": st["rounds"],
        "served_pair_steps": st["served_pair_steps"],
        "served_pair_steps_per_s": st["served_pair_steps"] / elapsed if elapsed > 0 else 0.0,
        "gpu_busy_fraction": st["kernel_ms"] * 1e-3 / elapsed if elapsed > 0 else 0.0,
        "setup_share_of_work": (st["setup_units"] / (st["setup_units"] + st["served_pair_steps"])
                                if st["setup_units"] + st["served_pair_steps"] else 0.0),
        "p50_s": _pct(lat, 50), "p99_s": _pct(lat, 99), "mean_s": float(np.mean(lat)) if lat else None,
        "p50_all_lower_bound_s": _pct(ages, 50), "p99_all_lower_bound_s": _pct(ages, 99),
    }
    if pair_steps_of is not None:
        arrived = [pair_steps_of(r) for k, (_, r) in enumerate(reqs[:submitted])]
        summary["offered_pair_steps"] = float(sum(arrived))
        summary["offered_pair_steps_per_s"] = float(sum(arrived)) / max(min(elapsed, reqs[-1][1][0]), 1e-9)
    return summary, done
