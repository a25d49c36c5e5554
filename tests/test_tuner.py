"""The native tuner (fs_autotune, fs_autotune_batch): it times launch shapes
on a sample, applies the fastest, caches the choice per GPU and workload
bucket, and never changes results."""
import os

import pytest

from factsieve_gb300 import tuner

pytestmark = pytest.mark.gpu

# a run long enough to tune (its samples take about a tenth of it)
LONG = (10**12, 10**12 + 3 * 10**10, 100_000, 200_000)
CHECK = (10**12, 10**12 + 3_000_000, 100_000, 200_000)


def test_tuned_search_gives_identical_results_and_is_cached(ctx, tmp_path):
    cache = str(tmp_path / "tuning.txt")
    base = ctx.sieve(*CHECK)
    best = tuner.autotune(ctx, *LONG, target_ms=500, cache_path=cache)
    try:
        assert best["shapes_tried"] >= 6 and best["rate"] > 0 and not best["from_cache"]
        t = best["tuning"]
        assert t["sieve_variant"] in (3, 5) and t["sieve_block_threads"] in (128, 256)
        assert ctx.tuning()["sieve_variant"] == t["sieve_variant"]        # applied to the context
        assert 1e5 <= best["seg_width"] <= 4_294_900_000
        assert best["steps_per_launch"] in (100_000, 99_992, 50_000)       # one launch, the check apart, halves
        tuned = ctx.sieve(*CHECK, seg_width=best["seg_width"])
        assert (tuned.raw_sum, tuned.primecount, tuned.checksum) == (base.raw_sum, base.primecount, base.checksum)
        # the same bucket again: read from the cache, nothing timed
        again = tuner.autotune(ctx, 10**12 + 7, 10**12 + 4 * 10**10, 100_003, 200_003, cache_path=cache)
        assert again["from_cache"] == 1 and again["shapes_tried"] == 0
        assert again["tuning"] == best["tuning"]
        # the split is cached against the n-width: the same choice for a
        # narrower n-range of the bucket
        other = tuner.autotune(ctx, 10**12 + 7, 10**12 + 4 * 10**10, 100_000, 190_000, cache_path=cache)
        assert other["from_cache"] == 1
        split = {100_000: 0, 99_992: 89_992, 50_000: 45_000}[best["steps_per_launch"]]
        assert other["tuning"]["max_steps_per_launch"] == split
        lines = open(cache).read().splitlines()
        assert len(lines) == 1 and lines[0].startswith("search|")
    finally:
        ctx.set_tuning()


def test_a_short_run_keeps_the_defaults(ctx, tmp_path):
    """A search whose samples would be more than about a tenth of it is not
    timed: the default shape, a segment width from the planning rate."""
    cache = str(tmp_path / "tuning.txt")
    r = tuner.autotune(ctx, 10**12, 10**12 + 30_000_000, 100_000, 101_000, cache_path=cache)
    assert (r["shapes_tried"], r["rate"], r["from_cache"]) == (0, 0.0, 0)
    assert r["tuning"]["sieve_variant"] == 5 and r["tuning"]["max_steps_per_launch"] == 0
    assert 1e5 <= r["seg_width"] <= 30_000_000
    assert not os.path.exists(cache)                                 # nothing measured, nothing cached


@pytest.mark.parametrize("shape", [
    dict(sieve_variant=3, sieve_blocks_per_sm=6, sieve_block_threads=128),
    dict(sieve_variant=5, sieve_blocks_per_sm=16, sieve_block_threads=128),
    dict(sieve_variant=5, sieve_blocks_per_sm=2, sieve_block_threads=256, max_steps_per_launch=333),
    dict(sieve_variant=5, max_steps_per_launch=992),                  # the check in a launch of its own
])
def test_every_shape_the_tuner_tries_gives_identical_results(ctx, orc, shape):
    lo, hi, nmin, nmax = 10**12, 10**12 + 3_000_000, 100_000, 101_000
    want = orc.run(lo, hi, nmin, nmax)
    ctx.set_tuning(**shape)
    try:
        r = ctx.sieve(lo, hi, nmin, nmax)
    finally:
        ctx.set_tuning()
    assert (r.raw_sum, r.primecount, r.checksum) == (want["raw_sum"], want["primecount"], want["checksum"])


def test_tuned_batch_tile_gives_identical_results(ctx, tmp_path):
    jobs = [(10**9 + 7, 10**9 + 4_000_007, 5000, 6000), (10**12, 10**12 + 6_000_000, 100_000, 100_500),
            ((1 << 40) + 1, (1 << 40) + 2_000_001, 20_000, 22_000)]
    base = ctx.batch_sieve(jobs)
    cache = str(tmp_path / "tuning.txt")
    got = tuner.autotune_batch(ctx, jobs, scale_down=4, cache_path=cache)
    try:
        assert got["tile"] in (1024, 2048, 4096) and got["ms"] > 0
        assert ctx.tuning()["batch_tile_candidates"] == got["tile"]
        for tile in (1024, 2048, 4096):
            ctx.set_tuning(batch_tile_candidates=tile)
            res = ctx.batch_sieve(jobs)
            assert [(r.raw_sum, r.primecount, r.checksum) for r in res] == \
                [(r.raw_sum, r.primecount, r.checksum) for r in base]
        again = tuner.autotune_batch(ctx, jobs, scale_down=4, cache_path=cache)
        assert again == {"tile": got["tile"], "ms": 0.0}
    finally:
        ctx.set_tuning()


def test_tuning_values_are_checked(ctx):
    import factsieve_gb300 as fs
    for bad in (dict(sieve_block_threads=64), dict(sieve_variant=4), dict(batch_tile_candidates=512)):
        with pytest.raises(fs.FSError):
            ctx.set_tuning(**bad)
    ctx.set_tuning()
