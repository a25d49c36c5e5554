"""Autotuner: candidate generation, bucket cache, and (GPU) that a tuned
launch shape leaves results unchanged."""
import pytest

from factsieve_gb300 import tuner


class FakeCtx:
    sm_count = 152

    def __init__(self):
        self.t = {}

    def set_tuning(self, **kw):
        self.t = kw

    def tuning(self):
        v = self.t.get("sieve_variant", 3)
        return {"sieve_variant": v, "sieve_blocks_per_sm": {3: 3, 5: 8}[v]}


def test_autotune_picks_fastest_and_caches(tmp_path):
    cache = tuner.TuningCache(str(tmp_path / "t.json"))
    calls = []

    def timer(ctx, cfg, pmin, width, nmin, nmax):
        calls.append(cfg)
        return 100.0 * cfg["sieve_variant"] - cfg["sieve_blocks_per_sm"]   # best: variant 5 at 8 blocks

    ctx = FakeCtx()
    best = tuner.autotune(ctx, 10**12, 100_000, 200_000, gpu_name="X", cache=cache, timer=timer)
    assert (best["sieve_variant"], best["sieve_blocks_per_sm"]) == (5, 8)
    assert len(calls) == 4
    again = tuner.autotune(ctx, 10**12 + 5, 100_001, 200_003, gpu_name="X", cache=cache, timer=timer)
    assert len(calls) == 4 and again["sieve_variant"] == 5          # same bucket: cached
    tuner.autotune(ctx, 10**15, 100_000, 200_000, gpu_name="X", cache=cache, timer=timer)
    assert len(calls) == 8                                            # new p bucket: tuned again


def test_bucket_key_separates_workloads():
    a = tuner.bucket_key("GB300", 152, 10**12, 10**5, 2 * 10**5)
    assert a != tuner.bucket_key("GB300", 152, 2**63, 10**6, 10**6 + 10**4)
    assert a == tuner.bucket_key("GB300", 152, 10**12 + 10**9, 10**5 + 7, 2 * 10**5 + 7)


@pytest.mark.gpu
def test_tuned_shape_gives_identical_results(ctx, tmp_path):
    import torch
    cache = tuner.TuningCache(str(tmp_path / "t.json"))
    best = tuner.autotune(ctx, 10**12, 100_000, 101_000, gpu_name=torch.cuda.get_device_name(0),
                          sample_steps=2e9, cache=cache)
    assert best["rate"] > 0 and len(best["tried"]) == 4
    base = ctx.sieve(10**12, 10**12 + 3_000_000, 100_000, 101_000)
    tuner.apply(ctx, best)
    try:
        tuned = ctx.sieve(10**12, 10**12 + 3_000_000, 100_000, 101_000)
    finally:
        ctx.set_tuning()
    assert (tuned.raw_sum, tuned.primecount, tuned.checksum) == (base.raw_sum, base.primecount, base.checksum)
