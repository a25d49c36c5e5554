"""Every launch-wide walk step against the oracle.

For a segment's p-range and its largest multiplier, fs_walk_step picks one
residue step proven valid for every candidate of the launch (walk_for_range,
fs_kernels.cu).  Each case here is a seeded random range that selects one
step, about half of them with bounds at that step's edges (the k_max bound
46 k_max < 7 2^23 of the float-quotient steps, their window shift at 32, the
64-bit product limit, 2^31 / 2^36 / 2^63 in p).  The whole search runs with
both kernel builds and ragged segment widths, and its prime count, raw
residue sum, checksum and factor count equal the oracle's bit for bit.  The
stage-level path, which picks a step per candidate, is compared in
test_gpu_parity.py; the reference has one step for every range, the
Montgomery product (cl_sieve.cpp's iterate kernel).
"""
import math
import random

import pytest

KB = 1_276_526          # the float-quotient steps' largest multiplier

# step: (least bit length of p, largest bit length, least k_max, largest k_max, description)
STEPS = {
    6: (7, 30, 34, 1 << 21, "32-bit half-offset"),
    7: (31, 35, KB + 1, (1 << 25) - 1, "shifted-window half-offset 64-bit"),
    9: (38, 59, 300, 441_505, "float quotient, window from the least p"),
    10: (33, 62, 300, KB, "float quotient, k_max-aware window, s >= 32"),
    11: (31, 40, 300, KB, "float quotient, k_max-aware window, s <= 32"),
    12: (42, 62, 300, KB, "float quotient, k_max-aware window, 96-bit product"),
    4: (36, 45, KB + 1, 1 << 22, "half-offset lazy 64-bit"),
    1: (33, 35, 1 << 25, (1 << 26) - 1, "lazy 64-bit"),
    5: (42, 62, KB + 1, (1 << 26) - 1, "half-offset lazy 96-bit"),
    2: (34, 62, 1 << 26, (1 << 26) + (1 << 16), "lazy 96-bit"),
    13: (63, 63, 34, KB, "half-offset canonical 96-bit, float quotient"),
    8: (63, 63, KB + 1, (1 << 26) - 1, "half-offset canonical 96-bit"),
    3: (63, 63, 1 << 26, (1 << 26) + (1 << 16), "canonical 96-bit"),
}


def _edges(step, kmax):
    """p values at which the step's validity changes, for this k_max."""
    out = []
    if step in (10, 12):
        out.append(((1 << 68) - 1) // (23 * kmax))          # ceil(23 p k_max / 16) reaches 2^64
    if step in (12, 13):
        out.append(1 << 63)                                  # the float quotient's two 96-bit forms meet
    if step in (10, 11):
        out += [((1 << 56) * 16) // (23 * kmax), ((1 << 55) * 16) // (23 * kmax)]   # window shift 32
    if step in (4, 1):
        out.append((1 << 62) // kmax)                        # p k_max = 2^62
    return [e for e in out if (1 << 31) < e <= (1 << 63)]


def _cases(step, count, seed):
    import factsieve_gb300 as fs
    bmin, bmax, kmin, kmax_hi, _ = STEPS[step]
    rng = random.Random(seed * 131 + step)
    out = []
    tries = 0
    while len(out) < count:
        tries += 1
        assert tries < 100_000, step
        kmax = rng.choice([rng.randrange(kmin, kmax_hi + 1), kmax_hi - rng.randrange(0, 2000),
                           int(math.exp(rng.uniform(math.log(kmin), math.log(kmax_hi))))])
        kmax = max(kmin, min(kmax, kmax_hi))
        w = rng.randrange(1000, 4000) if kmax >= 1 << 22 else rng.randrange(2000, 60_000)   # oracle time
        bits = rng.randrange(bmin, bmax + 1)
        edges = _edges(step, kmax)
        pick = rng.randrange(4)
        if pick == 0 and edges:
            e = rng.choice(edges)
            lo = rng.choice([e - w + rng.randrange(-3, 4), e + rng.randrange(-3, 4)])
        elif pick == 1:
            lo = (1 << bits) + rng.randrange(0, 50)          # at a power of two from above
        elif pick == 2:
            lo = (1 << (bits + 1)) - w - rng.randrange(0, 50)   # up to one from below
        else:
            lo = rng.randrange(1 << bits, 1 << (bits + 1))
        lo = max(lo, 3)
        hi = min(lo + w, (1 << 64) - 1)
        nmin = max(34, kmax - rng.randrange(1, 1500))
        if lo < nmin or fs.walk_step(lo, hi, kmax) != step:    # the search needs pmin >= nmin
            continue
        out.append((lo, hi, nmin, kmax))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("step", sorted(STEPS), ids=lambda s: f"step{s}")
def test_launch_wide_step_equals_the_oracle(ctx, orc, step):
    import factsieve_gb300 as fs
    rng = random.Random(step)
    bad = []
    cases = _cases(step, 8, 20261204)
    for variant in (5, 3):
        try:
            ctx.set_tuning(sieve_variant=variant)
            for lo, hi, nmin, nmax in cases:
                assert fs.walk_step(lo, hi, nmax) == step
                want = orc.run(lo, hi, nmin, nmax)
                assert want["status"] == 0
                r = ctx.sieve(lo, hi, nmin, nmax, seg_width=rng.choice([hi - lo, 7_777, 50_000]))
                if (r.primecount, r.raw_sum, r.checksum, r.factorcount) != \
                        (want["primecount"], want["raw_sum"], want["checksum"], want["factorcount"]):
                    bad.append((variant, lo, hi, nmin, nmax))
        finally:
            ctx.set_tuning()
    assert not bad, bad


def test_every_step_is_drawn_at_its_edges():
    """The case generator reaches each step (CPU: no search)."""
    for step in STEPS:
        cases = _cases(step, 8, 20261204)
        assert len(cases) == 8 and len(set(cases)) == 8
        assert all(nmin <= lo for lo, _, nmin, _ in cases)


# factors n! + c = 0 mod p with p just above 2^31 and n near the float-quotient
# steps' k_max bound (found by an oracle search of p in [2^31, 2^31 + 4e7),
# n in [1,270,000, 1,272,500]): the large-p ranges above have none
KNOWN_HITS = [(2147727289, -1270075), (2161892099, 1271298), (2163827261, 1272374),
              (2173926653, 1271794), (2179911557, 1271064), (2185959337, 1270653)]


def _factorial_mod(n, p):
    f = 1
    for k in range(2, n + 1):
        f = f * k % p
    return f


@pytest.mark.parametrize("p,nc", KNOWN_HITS[:2])
def test_known_hits_are_factors(p, nc):
    assert (_factorial_mod(abs(nc), p) + (-1 if nc < 0 else 1)) % p == 0


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [5, 3])
def test_float_quotient_step_reports_hits_near_the_kmax_bound(ctx, orc, variant):
    """Each window around a known factor runs the s <= 32 float-quotient step
    with multipliers up to 700 past the factor's n, and finds it."""
    import factsieve_gb300 as fs
    bad = []
    try:
        ctx.set_tuning(sieve_variant=variant)
        for p, nc in KNOWN_HITS:
            lo, hi, nmin, nmax = p - 3000, p + 3001, abs(nc) - 700, abs(nc) + 700
            assert fs.walk_step(lo, hi, nmax) == 11
            want = orc.run(lo, hi, nmin, nmax)
            r = ctx.sieve(lo, hi, nmin, nmax)
            got = [(int(q), int(n)) for q, n in zip(r.factors["p"], r.factors["nc"])]
            if (r.primecount, r.raw_sum, r.checksum) != (want["primecount"], want["raw_sum"], want["checksum"]) \
                    or got != [(p, nc)]:
                bad.append((p, nc, got))
    finally:
        ctx.set_tuning()
    assert not bad, bad
