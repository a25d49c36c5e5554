"""Launch-shape tuning: a thin front end of the library's native tuner.

fs_autotune (include/factsieve.h) times whole segment searches of a sample
of the real workload for each launch shape -- candidates per thread
(sieve_variant 3 or 5), blocks per SM (1x, 2x, 4x the resident ones),
threads per block (256 or 128), n-steps per launch (all, or halves) --
applies the fastest to the context and sizes a segment to a target kernel
time at the measured rate: the role of the reference's profileGPU
(cl_sieve.cpp:617-718) and of its setup/iterate retuning
(cl_sieve.cpp:1158-1227).  fs_autotune_batch picks the batch kernel's tile
size for a job mix.  Choices are cached in a text file (default
$FS_TUNING_CACHE, else ~/.cache/factsieve_gb300/tuning.txt) keyed by GPU
name, SM count and the workload's bucket.  Tuning never changes results.
"""
from __future__ import annotations

import os

__all__ = ["DEFAULT_CACHE", "autotune", "autotune_batch"]

DEFAULT_CACHE = os.environ.get("FS_TUNING_CACHE",
                               os.path.join(os.path.expanduser("~"), ".cache", "factsieve_gb300", "tuning.txt"))


def _dir_of(path):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    return path


def autotune(ctx, pmin, pmax, nmin, nmax, target_ms=1000.0, cache_path=DEFAULT_CACHE) -> dict:
    """Tune ctx for the search [pmin, pmax) x [nmin, nmax); returns the shape,
    the measured rate and the segment width (see Context.autotune)."""
    return ctx.autotune(pmin, pmax, nmin, nmax, target_ms, _dir_of(cache_path) if cache_path else None)


def autotune_batch(ctx, jobs, scale_down=16, cache_path=DEFAULT_CACHE) -> dict:
    """Tune the batch kernel's tile size for a job mix (see Context.autotune_batch)."""
    return ctx.autotune_batch(jobs, scale_down, _dir_of(cache_path) if cache_path else None)
