"""Throughput benchmark of the FactSieve GPU sieve: (p,n) pair-steps per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config3|config1]

Workload (default config2, the plain large sieve): p in [1e12, 1e12 + 1e9),
n in [1e5, 2e5).  One step = one pass over the whole p-range as one segment
(the command line's default segment width; wider segments leave a shorter
partial last wave), run through getsegprimes -> setup -> iterate -> check.
Config 3 passes run as 1e8-wide segments (its measured best); --segment
overrides the width (the ncu full capture uses 1e8).  After the timed
region, a one-GPU config2 run adds sub-objects for config 1 (end to end,
against its fixture), config 3 (one timed pass, roofline, e2e) and config 4
(the 64-job batch against 64 sequential plain runs); --no-extra skips them.
Metric: (p,n) pair-steps/s = candidates x (nmax - nmin) / time, plus the
fraction of the integer-multiply roofline.

  value      device-resident: the segment loop on one stream, CUDA events
             around the K timed steps, L2 flushed (256 MiB write) between
             steps; inputs (range, power table) are already on the device.
  e2e        the public API as a user calls it (Context.sieve on each step's
             segment): power table built on the host and uploaded, kernels,
             counters and hits copied back, CPU verification; wall clock.
  roofline   the dominant kernel (the fused setup/iterate/check sieve
             kernel) from CUDA events recorded around each of its launches on
             its stream, against the time its walk steps and setup products
             take at their measured ceilings (the same PTX blocks and
             Montgomery product register-resident at full occupancy); the
             reference's own accounting (20 IMAD per Montgomery product) and
             the HBM fraction are reported beside it.
  cpu_baseline  the CPU oracle (OpenMP over all host cores, the reference's
             algorithm restated) on a bounded slice of the same workload.

With --gpus N (torchrun, one rank per GPU) each rank takes a contiguous
share of the p-range (strong scaling: the whole range is one step at every
N); nothing crosses ranks on the data path, and the shares' raw sums and
candidate counts, added on the host, must equal the oracle fixture of the
whole range (the line's combined_check).

--impl reference times the reference's algorithm on the host CPU (the
oracle port: the reference's own GPU path is OpenCL and has no runtime
here) on a bounded slice per step, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (pmin, pmax, nmin, nmax, segment width)
    "config1": (1_000_000, 2_000_000, 1000, 2000, 1_000_000),      # a step is the whole (small) range
    "config2": (1_000_000_000_000, 1_001_000_000_000, 100_000, 200_000, 1_000_000_000),   # a step: the whole range
    "config3": (1 << 63, (1 << 63) + 1_000_000_000, 1_000_000, 1_010_000, 100_000_000),
}
IMAD_PER_PRODUCT = 20   # reference m_mul on 32-bit limbs (8 mul_wide + 4 + 8)
# DRAM bytes (read + write) per sieve launch and the integer-multiply pipe's
# busy share, from one `ncu --set full --clock-control none` capture of the
# fused sieve kernel on the same workload (dram__bytes_read.sum +
# dram__bytes_write.sum; sm__pipe_fmaheavy_cycles_active): config 2 captured
# on a 1e8-wide segment (29,087,744 B) and scaled by 10 to the whole-range
# launch the bench times, config 3 on one of its 1e8-wide launches.
NCU_CAPTURE = {   # workload -> sieve launches per segment -> capture
    "config2": {1: {"traffic": 290_877_440, "imad_pipe_busy": 0.785,
                    "source": "ncu --set full capture of sieve_kernel, bench.py --segment 1e8 --max-steps 0"},
                # the n-range in two launches: both launches of one 1e8-wide segment
                # (29,672,960 and 73,291,520 B), averaged and scaled by 10; the first
                # launch's 43 MB of residue state was still in L2 when it ended
                2: {"traffic": 514_822_400, "imad_pipe_busy": 0.783,
                    "source": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum of both sieve_kernel "
                              "launches, bench.py --segment 1e8 --max-steps 50000"}},
    "config3": {1: {"traffic": 18_705_664, "imad_pipe_busy": 0.851,
                    "source": "ncu --set full capture of sieve_kernel, bench.py --workload config3"}},
}
GOLDEN = os.path.join(ROOT, "tests", "golden")


# ------------------------------------------------------------ helpers -----

def reference_setup_products(nmin: int) -> int:
    """Montgomery products per candidate that the reference's setup kernel
    spends for nmin! (setup.cl:56-102 over the table of cl_sieve.cpp:818-835)."""
    import factsieve_gb300 as fs
    tp, te, tb = fs.power_table(nmin)
    prod = int(max(int(te[0]), 1).bit_length() - 1)          # entry 0: squarings (doublings are adds)
    for e in te[1:].tolist():
        prod += 2                                            # to Montgomery form + accumulate
        if e > 1:
            prod += (e.bit_length() - 1) + (bin(e).count("1") - 1)
    return prod


# Ceiling microkernels (fs_bench_int_pipe kinds) of each residue step.
STEP_CEILING_KIND = {6: (11, "32-bit half-offset step"), 7: (12, "shifted-window half-offset 64-bit step"),
                     9: (14, "half-offset 64-bit step, quotient on the FP32 pipe"),
                     10: (16, "half-offset 64-bit step, FP32 quotient over a k_max-sized window, s >= 32"),
                     11: (17, "half-offset 64-bit step, FP32 quotient over a k_max-sized window, s <= 32"),
                     12: (18, "half-offset 96-bit step, FP32 quotient over a k_max-sized window"),
                     13: (19, "half-offset canonical 96-bit step, FP32 quotient over a k_max-sized window"),
                     4: (5, "half-offset lazy 64-bit step"),
                     5: (10, "half-offset lazy 96-bit step"), 8: (13, "half-offset canonical 96-bit step"),
                     1: (6, "lazy 64-bit step"),
                     2: (7, "lazy 96-bit step"), 3: (8, "canonical 96-bit step"),
                     0: (9, "generic Montgomery step")}


def setup_products(fs, nmin: int, folded: bool = False):
    """Products per candidate outside the walk, as (plan products, other
    Montgomery products).  The bit-layered plan costs one product per word and
    one squaring per layer after the first; with Montgomery products the
    R^(D+1) correction (square-and-multiply over the deficit D) follows, while
    the folding products modulo 2^63 + d (folded=True) have no deficit but
    double by a product (one per doubling layer) and end with one conversion
    to Montgomery form.  Both add the constants R mod p and R^2 mod p (five
    squarings, built twice for four-candidate threads), entering and leaving
    the walk's residue form and the final nmax check."""
    words, layers, deficit = fs.setup_plan(nmin)
    plan = len(words) + max(len(layers) - 1, 0)
    if folded:
        return plan + int(sum(int(l[2]) for l in layers)), 1 + 10 + 2 + 3
    pow_d = max(int(deficit).bit_length() - 1, 0) + bin(int(deficit)).count("1")
    return plan, pow_d + 1 + 10 + 2 + 3


def roofline(ctx, fs, wl, ncand, st, step_ms, clocks=None, seg=None, segments=1):
    """Roofline of the fused sieve kernel.  The work is 64-bit modular
    multiplication: integer multiply-add, no memory traffic to speak of (the
    candidate list is read once).  The ceiling is the same arithmetic run
    register-resident at full occupancy on this GPU (fs_bench_int_pipe kinds
    4-15: the walk's own PTX step blocks, the Montgomery product and the
    folding product), so peak = pair-steps the kernel would finish if its walk
    ran at the walk ceiling and its setup products at their ceilings."""
    pmin, pmax, nmin, nmax, seg0 = WORKLOADS[wl]
    seg = seg or seg0
    W = nmax - nmin
    step = fs.walk_step(pmin, min(pmin + seg, pmax), nmax)
    kind, step_name = STEP_CEILING_KIND[step]
    walk_ceil, _ = ctx.bench_int_pipe(kind, 4000)
    mm_ceil, _ = ctx.bench_int_pipe(4, 4000)
    imad_ops, _ = ctx.bench_int_pipe(0, 20000)
    folded = bool(fs.setup_form(pmin, min(pmin + seg, pmax))) and step in (3, 8, 13)
    # the folding product's own ceiling is below Montgomery's at full occupancy
    # (it wins inside the fused kernel, at 2 blocks per SM): the peak takes the
    # faster of the two, so it never rests on the slower form
    fold_ceil = ctx.bench_int_pipe(15, 4000)[0] if folded else None
    plan_ceil = max(fold_ceil, mm_ceil) if folded else mm_ceil
    plan_products, mont_products = setup_products(fs, nmin, folded)
    smp = plan_products + mont_products
    sieve_s = st["sieve_ms"] * 1e-3
    launches = max(st["sieve_launches"], 1)
    pairs = ncand * W
    lower_bound_s = ncand * (W / walk_ceil + plan_products / plan_ceil + mont_products / mm_ceil)
    achieved = pairs / sieve_s if sieve_s > 0 else 0.0
    peak = pairs / lower_bound_s if lower_bound_s > 0 else 0.0
    # launches per pass: 1 (setup, walk and check fused) or L > 1 when the n-range
    # is split (the tuner's choice); each launch reads the candidate list, and
    # between launches every candidate's residue and walked-n tag (12 bytes)
    # are written and read back
    per_pass = max(int(round(launches / max(segments, 1))), 1)
    cap = NCU_CAPTURE.get(wl, {}).get(per_pass, {})
    alg_bytes = (8.0 * per_pass + 24.0 * (per_pass - 1)) * ncand / launches
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    hbm_ach = alg_bytes / (sieve_s / launches) / 1e9 if sieve_s > 0 else 0.0
    # the reference's own accounting (a 20-IMAD Montgomery product per step and
    # per setup product): reference-equivalent products against IMAD rate / 20
    ref_products = ncand * (W + reference_setup_products(nmin) + 1)
    ref_peak = imad_ops / IMAD_PER_PRODUCT
    sm = (clocks or {}).get("sm_mhz") or 0
    sm_max = (clocks or {}).get("sm_max_mhz") or 0
    return {
        "bound": "imad", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "G pair-steps/s",
        "frac": achieved / peak if peak else None,
        "traffic": cap.get("traffic"), "algorithmic_bytes_per_launch": alg_bytes,
        "launches_per_segment": per_pass,
        "kernel": "sieve_kernel (setup + walk + check fused)",
        "kernel_ms_per_launch": st["sieve_ms"] / launches,
        "share_of_step": st["sieve_ms"] / step_ms if step_ms else None,
        "walk_step": step_name,
        "ceilings": {"walk_steps_per_s": walk_ceil, "montgomery_products_per_s": mm_ceil,
                     "folding_products_per_s": fold_ceil, "plan_products_per_s": plan_ceil,
                     "imad_lane_ops_per_s": imad_ops},
        "setup_products_per_candidate": smp,
        "setup_product": "folding modulo 2^63 + d" if folded else "Montgomery",
        "peak_source": "measured on this GPU: the walk step's PTX block and mont_mul, register-resident at full "
                       "occupancy (fs_bench_int_pipe kinds 4-19)",
        "imad_pipe_busy_ncu": cap.get("imad_pipe_busy"), "ncu_source": cap.get("source"),
        "hbm": {"achieved": hbm_ach, "peak": hbm_peak, "unit": "GB/s",
                "frac": hbm_ach / hbm_peak if hbm_peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s"},
        "reference_mulmod_roofline": {
            "achieved": ref_products / sieve_s / 1e9 if sieve_s > 0 else 0.0,
            "peak": ref_peak / 1e9, "unit": "G Montgomery products/s",
            "frac": (ref_products / sieve_s) / ref_peak if sieve_s > 0 else None,
            "iterate_only_frac": (pairs / sieve_s) / ref_peak if sieve_s > 0 else None,
            "peak_at_max_clock": ref_peak / 1e9 * (sm_max / sm) if sm and sm_max else None,
            "definition": "reference-equivalent products (one per (p,n) step plus the reference setup's table "
                          "products and one check) / (measured IMAD rate / 20 IMAD per product), at the sampled "
                          "clock; iterate_only counts the walk steps alone"},
    }


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for k, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    import torch.distributed as dist
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist if ws > 1 else None


# ------------------------------------------------------------ CPU legs ----

def cpu_slice_run(pmin, nmin, nmax, width):
    """The oracle (reference algorithm on the CPU) over [pmin, pmin + width)."""
    import oracle
    oracle.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    r = oracle.run(pmin, pmin + width, nmin, nmax, seg_width=width)
    dt = time.perf_counter() - t0
    return r, dt


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo; on Arm the implementer and part)."""
    try:
        with open("/proc/cpuinfo") as fh:
            info = fh.read()
    except OSError:
        return "unknown"
    for key in ("model name", "Model", "CPU part"):
        for line in info.splitlines():
            if line.startswith(key):
                val = line.split(":", 1)[1].strip()
                if key == "CPU part":
                    impl = next((ln.split(":", 1)[1].strip() for ln in info.splitlines()
                                 if ln.startswith("CPU implementer")), "?")
                    return f"implementer {impl} part {val}"
                return val
    return "unknown"


def cpu_baseline(wl, budget_s=40.0):
    """The oracle on all host cores: config 1 in full, configs 2 and 3 on the
    fixed contiguous 1/100 slice at the start of the p-range (the work is
    uniform in p, so pair-steps/s carry over), shrunk only if a probe says the
    slice would take longer than budget_s."""
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    width = pmax - pmin if wl == "config1" else (pmax - pmin) // 100
    probe = max(20_000, min(width, 200_000))
    r, dt = cpu_slice_run(pmin, nmin, nmax, probe)
    est = dt * width / probe
    label = "the whole range" if wl == "config1" else "the fixed 1/100 slice"
    if est > budget_s:
        width = int(max(probe, width * budget_s / est))
        label = f"a {width}-wide slice (the 1/100 slice would take ~{est:.0f} s)"
    r, dt = cpu_slice_run(pmin, nmin, nmax, width)
    pairs = r["primecount"] * (nmax - nmin)
    return {"value": pairs / dt, "unit": "pair-steps/s", "cores": os.cpu_count(), "kind": "port",
            "cpu": cpu_model(),
            "sample": f"{label}: p in [{pmin}, {pmin + width}) ({r['primecount']} candidates, "
                      f"n in [{nmin}, {nmax})), oracle/oracle.c OpenMP, {dt:.1f} s"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    wl = args.workload
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    import oracle
    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    # bounded per-step sample of the workload: consecutive slices of the range
    width = {"config1": 100_000, "config2": 1_000_000, "config3": 1_000_000}[wl]
    for i in range(args.warmup):
        cpu_slice_run(pmin + i * width, nmin, nmax, width)
    pairs = 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        r, _ = cpu_slice_run(pmin + (args.warmup + i) * width, nmin, nmax, width)
        pairs += r["primecount"] * (nmax - nmin)
    dt = time.perf_counter() - t0
    value = pairs / dt
    line = {
        "metric": "(p,n) pair-steps/sec", "value": value, "unit": "pair-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"{wl}: p in [{pmin}, {pmax}), n in [{nmin}, {nmax})",
                   "step": f"a {width}-wide slice of the p-range per step (bounded CPU sample)",
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "pair-steps/s", "cores": os.cpu_count(), "kind": "port",
                         "cpu": cpu_model(),
                         "sample": f"{args.steps} consecutive {width}-wide p-slices, oracle/oracle.c OpenMP "
                                   f"(the reference's OpenCL path has no runtime on this host)"},
        "e2e": {"value": value, "unit": "pair-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ GPU leg -----

def fixture(wl):
    """The oracle's result for the whole workload range (tests/golden/run_<wl>.json)."""
    try:
        with open(os.path.join(GOLDEN, f"run_{wl}.json")) as fh:
            d = json.load(fh)
    except OSError:
        return None
    return {"raw_sum": int(d["raw_sum"], 16), "primecount": int(d["primecount"])}


def run_ours(args):
    import torch
    import factsieve_gb300 as fs
    from factsieve_gb300.shard import shard_bounds
    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    dist = init_dist(ws, "nccl" if ws > 1 else None)
    wl = args.workload
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    if args.segment:
        seg = int(args.segment)
    W = nmax - nmin
    # my contiguous share of the whole range; one step = my share, as segments of width seg
    lo, hi = shard_bounds(pmin, pmax, ws, rank)
    segs = [(a, min(a + seg, hi)) for a in range(lo, hi, seg)]

    ctx = fs.Context(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2

    def one_step():
        for s_lo, s_hi in segs:
            ctx.segment(s_lo, s_hi)

    # the launch shape: measured on a sample of this rank's share by the
    # library's tuner (fs_autotune) and applied to the context, tuned for the
    # work of a run of at least 20 passes over the share (its samples take
    # about a tenth of that; the tuning is outside the timed region)
    passes = max(args.warmup + args.steps, 20)
    tune = ctx.autotune(lo, min(lo + (hi - lo) * passes, (1 << 64) - 1), nmin, nmax)
    if args.max_steps is not None:
        # a fixed n-range split (0: one launch per segment) over the tuned shape, for captures
        t = dict(tune["tuning"], max_steps_per_launch=args.max_steps)
        ctx.set_tuning(**t)
        tune["tuning"] = t
    ctx.begin(pmin, pmax, nmin, nmax)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            one_step()
            flush.fill_(1)
    cap = 30_000_000 if pmin < 0xFFFFFFFF else 1_000_000
    ctx.collect(cap)                       # drain warm-up work and counters
    ctx.reset_stats()
    ctx.set_timing(True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(stream):
            e0.record(stream)
            for j in range(args.steps):
                one_step()
                if j + 1 < args.steps:
                    flush.fill_(j & 0xFF)  # L2 flush between timed steps
            e1.record(stream)
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    st = ctx.stats()
    ctx.set_timing(False)
    hits, raw, primecount, flags, rc = ctx.collect(cap)
    assert rc == 0, f"device flagged {flags}"
    my_pc = primecount
    pairs = primecount * W
    # max time over ranks, total work over ranks; the shares' sums combine on the host
    # (u64 adds), and K passes over the whole range must give K times its oracle result
    shares = [(raw, primecount)]
    if dist:
        t = torch.tensor([ms, float(pairs)], dtype=torch.float64, device=dev)
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = t.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        ms, pairs = tmax[0].item(), tsum[1].item()
        shares = [None] * ws
        dist.all_gather_object(shares, (raw, primecount))
    M = (1 << 64) - 1
    comb_raw = sum(r for r, _ in shares) & M
    comb_pc = sum(c for _, c in shares)
    primecount = comb_pc
    want = fixture(wl)
    check = None
    if want:
        K = args.steps
        check = {"combined_raw_sum": f"{comb_raw:016X}", "combined_primecount": comb_pc,
                 "expected_raw_sum": f"{(want['raw_sum'] * K) & M:016X}",
                 "expected_primecount": want["primecount"] * K,
                 "source": f"tests/golden/run_{wl}.json (oracle), times {K} timed passes",
                 "equal": comb_raw == (want["raw_sum"] * K) & M and comb_pc == want["primecount"] * K}
    value = pairs / (ms * 1e-3)

    # roofline of the dominant kernel, from this rank's events
    roof = roofline(ctx, fs, wl, my_pc, st, ms, clk.summary(), seg, segments=len(segs) * args.steps)
    # e2e through the public API with host buffers: every rank searches its
    # whole share with Context.sieve per step (plan upload, counters and hits
    # back, CPU verification), wall clock, max over ranks
    e2e_steps = max(1, min(args.steps, 3))
    ctx.set_stream(None)
    words, layers, _ = fs.setup_plan(nmin)          # the plan each call uploads (bytes counted below)
    plan_bytes = words.nbytes + layers.nbytes
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_pairs = 0
    h2d = d2h = 0
    for _ in range(e2e_steps):
        r = ctx.sieve(lo, hi, nmin, nmax, threads=os.cpu_count() or 2)
        e2e_pairs += r.primecount * W
        h2d += plan_bytes + 64
        d2h += 32 + 16 * r.nhits
    dt = time.perf_counter() - t0
    if dist:
        t = torch.tensor([dt, float(e2e_pairs)], dtype=torch.float64, device=dev)
        tmax, tsum = t.clone(), t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        dt, e2e_pairs = tmax[0].item(), tsum[1].item()
    e2e = {"value": e2e_pairs / dt, "unit": "pair-steps/s", "h2d_bytes_per_step": h2d // e2e_steps,
           "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps,
           "path": "Context.sieve (fs_search_begin/segment/collect + fs_postprocess) on each rank's share"}
    # the reference accounting end to end: e2e pair-steps/s with each step's
    # share of the reference's setup and check products
    ref = roof["reference_mulmod_roofline"]
    per_step = (W + reference_setup_products(nmin) + 1) / W
    ref["end_to_end_frac"] = e2e["value"] * per_step / ws / (ref["peak"] * 1e9) if ref["peak"] else None

    if rank == 0:
        cpu = cpu_baseline(wl) if (ws == 1 and not args.no_cpu) else None
        line = {
            "metric": "(p,n) pair-steps/sec", "value": value, "unit": "pair-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (integer ranges; no dataset)",
            "config": {"workload": f"{wl}: p in [{pmin}, {pmax}), n in [{nmin}, {nmax})",
                       "step": f"one pass over the whole p-range: each rank its contiguous share, as "
                               f"{len(segs)} segment(s) of up to {seg}",
                       "parallelism": f"contiguous p-shares over {ws} GPU(s), no collective on the data path; "
                                      f"the shares' sums combine on the host",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "candidates_timed": primecount, "pair_steps_timed": pairs},
            "combined_check": check,
            "tuning": {"shape": tune["tuning"], "sample_rate_pair_steps_per_s": tune["rate"],
                       "shapes_tried": tune["shapes_tried"], "by": "fs_autotune on a sample of the share"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(st["launches"]),
            "clocks": clk.summary(),
        }
        if ws == 1 and wl == "config2" and not args.no_extra:
            # the other single-GPU configurations, after the timed region
            line["config1"] = extra_config1(ctx, fs)
            line["config3"] = extra_config3(ctx, fs, torch, dev)
            line["config4"] = batch_compare(ctx, fs, torch, dev, load_jobs(), warmup=1)
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def extra_config1(ctx, fs):
    """Config 1 (p in [1e6, 2e6), n in [1000, 2000)) through Context.sieve,
    wall clock, against its oracle fixture."""
    pmin, pmax, nmin, nmax, _ = WORKLOADS["config1"]
    ctx.set_stream(None)
    ctx.set_tuning()                                   # default shapes (too small a run to time)
    ctx.sieve(pmin, pmax, nmin, nmax)                  # warm-up
    t0 = time.perf_counter()
    r = ctx.sieve(pmin, pmax, nmin, nmax, threads=os.cpu_count() or 2)
    dt = time.perf_counter() - t0
    with open(os.path.join(GOLDEN, "run_config1.json")) as fh:
        want = json.load(fh)
    return {"workload": f"config1: p in [{pmin}, {pmax}), n in [{nmin}, {nmax})",
            "e2e_pair_steps_per_s": r.primecount * (nmax - nmin) / dt, "wall_s": dt,
            "primecount": r.primecount, "factorcount": r.factorcount, "checksum": f"{r.checksum:016X}",
            "equals_oracle_fixture": (r.primecount, r.factorcount, f"{r.checksum:016X}") ==
                                     (want["primecount"], want["factorcount"], want["checksum"])}


def extra_config3(ctx, fs, torch, dev):
    """Config 3 (p in [2^63, 2^63 + 1e9), n in [1e6, 1.01e6)): one untimed and
    one timed pass over the whole range as 1e8-wide segments on the library's
    stream (CUDA events around the pass and around each sieve launch), the
    kernel's roofline against its ceilings, and one 1e8-wide segment end to end
    through Context.sieve."""
    wl = "config3"
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    W = nmax - nmin
    segs = [(a, min(a + seg, pmax)) for a in range(pmin, pmax, seg)]
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # tuned as for a 20-pass run of this workload (the two passes below alone
    # are too short for the tuner to spend its samples on)
    tune = ctx.autotune(pmin, pmin + (pmax - pmin) * 20, nmin, nmax)
    ctx.begin(pmin, pmax, nmin, nmax)
    with torch.cuda.stream(stream):
        for s_lo, s_hi in segs:
            ctx.segment(s_lo, s_hi)
        flush.fill_(3)
    ctx.collect(1 << 20)
    ctx.reset_stats()
    ctx.set_timing(True)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        with torch.cuda.stream(stream):
            e0.record(stream)
            for s_lo, s_hi in segs:
                ctx.segment(s_lo, s_hi)
            e1.record(stream)
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    st = ctx.stats()
    ctx.set_timing(False)
    _, raw, pc, flags, rc = ctx.collect(1 << 20)
    want = fixture(wl)
    roof = roofline(ctx, fs, wl, pc, st, ms, clk.summary(), seg, segments=len(segs))
    ctx.set_stream(None)
    t0 = time.perf_counter()
    r = ctx.sieve(segs[0][0], segs[0][1], nmin, nmax, threads=os.cpu_count() or 2)
    dt = time.perf_counter() - t0
    return {"workload": f"config3: p in [{pmin}, {pmax}), n in [{nmin}, {nmax})",
            "value": pc * W / (ms * 1e-3), "unit": "pair-steps/s", "ms_per_pass": ms,
            "step": f"one pass over the whole range as {len(segs)} segments of {seg}",
            "equals_oracle_fixture": (raw, pc, rc) == (want["raw_sum"], want["primecount"], 0) if want else None,
            "roofline": {k: roof[k] for k in ("bound", "achieved", "peak", "unit", "frac", "kernel_ms_per_launch",
                                              "walk_step", "setup_product", "setup_products_per_candidate",
                                              "ceilings")},
            "e2e": {"value": r.primecount * W / dt, "unit": "pair-steps/s", "wall_s": dt,
                    "path": f"Context.sieve over [{segs[0][0]}, {segs[0][1]})"},
            "tuning": {"shape": tune["tuning"], "shapes_tried": tune["shapes_tried"]},
            "clocks": clk.summary()}


def load_jobs():
    with open(os.path.join(GOLDEN, "jobs_config4.json")) as fh:
        return [tuple(j) for j in json.load(fh)["jobs"]]


def batch_compare(ctx, fs, torch, dev, jobs, warmup=3):
    """Config 4: the 64 uneven jobs (seed 1) in one persistent, graph-captured
    launch against the same 64 jobs run one after another through the plain
    path on the same GPU.  Both legs are timed with CUDA events on the
    library's stream (device time) and with the wall clock; every job's
    (primecount, raw sum, hits) must agree between the legs."""
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    cap = 1 << 20
    small = [(p0, p0 + max(10_000, (p1 - p0) // 200), n0, n1) for p0, p1, n0, n1 in jobs]
    for _ in range(warmup):                       # warm-up: the same mix at 1/200 of the p-widths
        ctx.batch_sieve(small)
    # the batch kernel's tile size, measured on the mix at 1/32 of its p-widths
    tile = ctx.autotune_batch(jobs, scale_down=32)
    # batched leg
    ctx.batch_prepare(jobs, hitcap=cap)
    ctx.reset_stats()
    ctx.set_timing(True)
    torch.cuda.synchronize(dev)
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        ctx.batch_launch()
        res, hits, rc = ctx.batch_collect()
        wall_b = time.perf_counter() - t0
    st = ctx.stats()
    ctx.set_timing(False)
    assert rc == 0
    dev_b = st["batch_ms"] * 1e-3
    pairs = sum(r["primecount"] * (j[3] - j[2]) for r, j in zip(res, jobs))
    ctx.batch_release()
    # plain leg: 64 sequential searches
    ctx.set_tuning()
    ctx.reset_stats()
    ctx.set_timing(True)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plain = []
    for j in jobs:
        ctx.begin(*j)
        ctx.run_range(j[0], j[1])
        h, raw, pc, flags, rc2 = ctx.collect(cap)
        assert rc2 == 0
        plain.append((pc, raw, sorted(zip(h["p"].tolist(), h["nc"].tolist()))))
    wall_p = time.perf_counter() - t0
    sp = ctx.stats()
    ctx.set_timing(False)
    ctx.set_stream(None)
    dev_p = (sp["sieve_ms"] + sp["gen_ms"]) * 1e-3
    same = True
    for k, (r, pl) in enumerate(zip(res, plain)):
        mine = sorted(zip(hits["p"][hits["pad"] == k].tolist(), hits["nc"][hits["pad"] == k].tolist()))
        same &= (r["primecount"], r["raw_sum"], mine) == pl
    return {"workload": "config4: 64 uneven jobs in one persistent launch (tests/golden/jobs_config4.json)",
            "pair_steps": pairs, "value": pairs / dev_b, "unit": "pair-steps/s",
            "batched": {"device_s": dev_b, "wall_s": wall_b, "pair_steps_per_s": pairs / dev_b,
                        "wall_pair_steps_per_s": pairs / wall_b, "launches": int(st["launches"])},
            "plain_sequential": {"device_s": dev_p, "wall_s": wall_p, "pair_steps_per_s": pairs / dev_p,
                                 "wall_pair_steps_per_s": pairs / wall_p, "launches": int(sp["launches"])},
            "speedup_device": dev_p / dev_b, "speedup_wall": wall_p / wall_b,
            "per_job_bit_exact": bool(same), "warmup": "the same 64 jobs at 1/200 of their p-widths",
            "tuning": {"batch_tile_candidates": tile["tile"], "sample_batch_ms": tile["ms"],
                       "by": "fs_autotune_batch on the mix at 1/32 of its p-widths; the plain leg runs default "
                             "shapes"},
            "clocks": clk.summary()}


def run_batch(args):
    """Config 4 as its own line (batch_compare)."""
    import torch
    import factsieve_gb300 as fs
    dev = torch.cuda.current_device()
    ctx = fs.Context(dev)
    b = batch_compare(ctx, fs, torch, dev, load_jobs(), warmup=args.warmup)
    line = {
        "metric": "(p,n) pair-steps/sec", "value": b["value"], "unit": "pair-steps/s", "n_gpus": 1,
        "steps": 1, "warmup": args.warmup, "ms_per_step": b["batched"]["device_s"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (64 jobs, seed 1)",
        "config": {"workload": b["workload"], "warmup": b["warmup"], "pair_steps": b["pair_steps"]},
        "batched": b["batched"], "plain_sequential": b["plain_sequential"],
        "speedup_device": b["speedup_device"], "speedup_wall": b["speedup_wall"],
        "per_job_bit_exact": b["per_job_bit_exact"],
        "gpu_launches": b["batched"]["launches"],
        "clocks": b["clocks"],
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_serve(args):
    """Config 5: the seed-2 Poisson stream (20 requests/s for 120 s, job sizes
    from the config-4 distribution) replayed in real time through the serving
    loop, reporting served versus offered load and p50/p99 sojourn time.  The
    offered load is far above one GPU, so a second, explicitly labelled run
    replays the same arrivals with every p-width divided by 1000."""
    import math
    import torch
    import factsieve_gb300 as fs
    from factsieve_gb300.serve import run_stream
    with open(os.path.join(GOLDEN, "stream_config5.json")) as fh:
        reqs = [tuple(r) for r in json.load(fh)["requests"]]
    dev = torch.cuda.current_device()
    ctx = fs.Context(dev)

    def est_pairs(r):
        p0, p1, n0, n1 = r[1:5] if len(r) == 5 else r
        return (p1 - p0) / math.log(p0) * (n1 - n0)

    # warm-up: three short streams
    small = [(t * 0.01, p0, p0 + max(10_000, (p1 - p0) // 2000), n0, n1) for t, p0, p1, n0, n1 in reqs[:20]]
    for _ in range(args.warmup):
        run_stream(ctx, small, stop_after_s=30)
    with ClockSampler(dev) as clk:
        full, done_full = run_stream(ctx, reqs, stop_after_s=args.serve_seconds, max_active=16,
                                     pair_steps_of=est_pairs)
    scaled = [(t, p0, p0 + max(10_000, (p1 - p0) // 1000), n0, n1) for t, p0, p1, n0, n1 in reqs]
    small_sum, done_small = run_stream(ctx, scaled, stop_after_s=args.serve_seconds, max_active=16,
                                       pair_steps_of=est_pairs)
    # bit-exactness of a sample of finished jobs against the same job alone
    sample = sorted(done_small)[:: max(1, len(done_small) // 8)][:8]
    exact = True
    for k in sample:
        d = done_small[k]
        _, p0, p1, n0, n1 = scaled[k]
        a = ctx.sieve(p0, p1, n0, n1, threads=os.cpu_count() or 2)
        kept, cs_add, _ = fs.postprocess(d["hits"], threads=os.cpu_count() or 2)
        exact &= (d["primecount"], (d["raw_sum"] + cs_add) & 0xFFFFFFFFFFFFFFFF) == (a.primecount, a.checksum)
    line = {
        "metric": "(p,n) pair-steps/sec", "value": full["served_pair_steps_per_s"], "unit": "pair-steps/s",
        "n_gpus": 1, "steps": 1, "warmup": args.warmup, "ms_per_step": full["elapsed_s"] * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (Poisson stream, seed 2)",
        "config": {"workload": "config5: Poisson 20 req/s for 120 s, config-4 job sizes, continuous batching",
                   "stop_after_s": args.serve_seconds, "max_active": 16},
        "served": full,
        "offered_vs_served": {"offered_pair_steps_per_s_est": full.get("offered_pair_steps_per_s"),
                              "served_pair_steps_per_s": full["served_pair_steps_per_s"]},
        "latency_s": {"p50": full["p50_s"], "p99": full["p99_s"],
                      "p50_all_lower_bound": full["p50_all_lower_bound_s"],
                      "p99_all_lower_bound": full["p99_all_lower_bound_s"],
                      "note": "sojourn (arrival to result) of completed requests; the stream overloads one GPU, "
                              "so later requests are still queued: the *_all_lower_bound figures count every "
                              "submitted request, an unfinished one at its age when the window closed"},
        "scaled_down_stream": dict(small_sum, label="same arrivals, every p-width divided by 1000"),
        "per_job_bit_exact_sample": {"jobs": len(sample), "exact": bool(exact)},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS) + ["config4", "config5"])
    ap.add_argument("--serve-seconds", type=float, default=180.0, help="config5: stop the replay after this long")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--max-steps", type=int, default=None,
                    help="override the tuned n-steps per launch (0: the whole n-range in one launch)")
    ap.add_argument("--no-extra", action="store_true",
                    help="config2 at one GPU: skip the config1/config3/config4 sub-objects after the timed region")
    ap.add_argument("--segment", type=float, default=0,
                    help="p-width of one step (default: the workload's; e.g. 1e8 for a short profiling case)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "config4":
        return run_batch(args)
    if args.workload == "config5":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
