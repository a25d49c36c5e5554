"""Autotuner for the sieve launch shape.

Knobs (fs_tuning in include/factsieve.h):
  sieve_variant         the sieve kernel build: 3 = two candidates per thread
                        at 3 resident 256-thread blocks per SM (register cap
                        85), 5 = four candidates per thread (two interleaved
                        pairs) at 2 blocks per SM
  sieve_blocks_per_sm   blocks launched per SM (beyond the resident ones they
                        run as later waves, which evens out the last wave)
  segment width         p-width of one launch (candidates per launch: larger
                        segments shorten the partial last wave)
The block size (256) is fixed in the kernels.

A configuration is timed on a short sample of the real workload with CUDA
events (fs_get_stats), the fastest wins, and the choice is cached in a JSON
file keyed by GPU, SM count and the workload's bucket: log2 of the n-width,
of p and of nmin.  The tuning never changes results, only speed.
"""
from __future__ import annotations

import json
import math
import os
import threading

__all__ = ["bucket_key", "TuningCache", "autotune", "apply"]

DEFAULT_CACHE = os.environ.get("FS_TUNING_CACHE",
                               os.path.join(os.path.expanduser("~"), ".cache", "factsieve_gb300", "tuning.json"))


def bucket_key(gpu: str, sms: int, pmin: int, nmin: int, nmax: int) -> str:
    w = max(nmax - nmin, 1)
    return f"{gpu}|sm{sms}|W{int(math.log2(w))}|P{int(math.log2(max(pmin, 2)))}|N{int(math.log2(max(nmin, 2)))}"


class TuningCache:
    """JSON file of bucket -> best configuration (thread-safe, atomic rewrite)."""

    def __init__(self, path: str = DEFAULT_CACHE):
        self.path = path
        self._lock = threading.Lock()

    def load(self) -> dict:
        try:
            with open(self.path) as fh:
                return json.load(fh)
        except (OSError, ValueError):
            return {}

    def get(self, key):
        return self.load().get(key)

    def put(self, key, value):
        with self._lock:
            data = self.load()
            data[key] = value
            os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
            tmp = self.path + ".tmp"
            with open(tmp, "w") as fh:
                json.dump(data, fh, indent=1, sort_keys=True)
            os.replace(tmp, self.path)


VARIANTS = (3, 5)


def candidates(default_blocks_by_variant):
    """Configurations to try: every variant at its default blocks per SM, and at 2x."""
    out = []
    for v, d in default_blocks_by_variant.items():
        out.append({"sieve_variant": v, "sieve_blocks_per_sm": d})
        out.append({"sieve_variant": v, "sieve_blocks_per_sm": 2 * d})
    return out


def _time_config(ctx, cfg, pmin, width, nmin, nmax):
    ctx.set_tuning(sieve_variant=cfg["sieve_variant"], sieve_blocks_per_sm=cfg["sieve_blocks_per_sm"])
    ctx.begin(pmin, pmin + 2 * width, nmin, nmax)
    ctx.segment(pmin, pmin + width)                   # warm-up (plan upload, table check)
    ctx.collect(1 << 20, raise_on_flags=True)
    ctx.reset_stats()
    ctx.set_timing(True)
    ctx.segment(pmin + width, pmin + 2 * width)
    st = ctx.stats()
    ctx.set_timing(False)
    _, _, pc, _, _ = ctx.collect(1 << 20)
    sec = (st["sieve_ms"] + st["gen_ms"]) * 1e-3
    return pc * (nmax - nmin) / sec if sec > 0 else 0.0


def autotune(ctx, pmin, nmin, nmax, gpu_name="gpu", sample_steps=2e10, cache: TuningCache | None = None,
             timer=None, force=False):
    """Best configuration for this workload bucket (cached).  `sample_steps` sizes
    the timing sample in (p,n) steps.  `timer(ctx, cfg, pmin, width, nmin, nmax)`
    replaces the GPU timing (tests)."""
    cache = cache or TuningCache()
    key = bucket_key(gpu_name, ctx.sm_count, pmin, nmin, nmax)
    if not force:
        hit = cache.get(key)
        if hit:
            return hit
    occ = {}
    for v in VARIANTS:
        ctx.set_tuning(sieve_variant=v)
        occ[v] = ctx.tuning()["sieve_blocks_per_sm"]
    per_cand = (nmax - nmin) + 0.1 * nmin + 64
    width = int(min(max(sample_steps / per_cand * math.log(max(pmin, 3)), 200_000), 2e9))
    timer = timer or _time_config
    best, best_rate = None, -1.0
    tried = []
    for cfg in candidates(occ):
        rate = timer(ctx, cfg, pmin, width, nmin, nmax)
        tried.append(dict(cfg, rate=rate))
        if rate > best_rate:
            best, best_rate = cfg, rate
    ctx.set_tuning()
    result = dict(best, rate=best_rate, sample_width=width, tried=tried)
    cache.put(key, result)
    return result


def apply(ctx, cfg) -> None:
    """Apply a configuration returned by autotune() to a Context."""
    ctx.set_tuning(sieve_variant=int(cfg["sieve_variant"]), sieve_blocks_per_sm=int(cfg["sieve_blocks_per_sm"]))
