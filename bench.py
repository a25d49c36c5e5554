"""Throughput benchmark of the FactSieve GPU sieve: (p,n) pair-steps per second.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config2|config3|config1]

Workload (default config2, the plain large sieve): p in [1e12, 1e12 + 1e9),
n in [1e5, 2e5).  One step = one p-segment of 1e8 (so 10 steps cover the
configuration once), run through getsegprimes -> setup -> iterate -> check.
Metric: (p,n) pair-steps/s = candidates x (nmax - nmin) / time, plus the
fraction of the IMAD-limited Montgomery-product roofline.

  value      device-resident: the segment loop on one stream, CUDA events
             around the K timed steps, L2 flushed (256 MiB write) between
             steps; inputs (range, power table) are already on the device.
  e2e        the public API as a user calls it (Context.sieve on each step's
             segment): power table built on the host and uploaded, kernels,
             counters and hits copied back, CPU verification; wall clock.
  roofline   the dominant kernel (the fused setup/iterate/check sieve
             kernel) from CUDA events recorded around each of its launches on
             its stream: reference-equivalent Montgomery products per second
             against the measured IMAD rate / 20 IMAD per product.
  cpu_baseline  the CPU oracle (OpenMP over all host cores, the reference's
             algorithm restated) on a bounded slice of the same workload.

With --gpus N (torchrun, one rank per GPU) the p-segments are dealt
round-robin to the ranks: no data-path collective, weak scaling.

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
    "config1": (1_000_000, 2_000_000, 1000, 2000, 100_000),
    "config2": (1_000_000_000_000, 1_001_000_000_000, 100_000, 200_000, 100_000_000),
    "config3": (1 << 63, (1 << 63) + 1_000_000_000, 1_000_000, 1_010_000, 100_000_000),
}
IMAD_PER_PRODUCT = 20   # reference m_mul on 32-bit limbs (8 mul_wide + 4 + 8)


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


def cpu_baseline(wl, budget_s=15.0):
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    # size the slice from a short probe so the measurement takes ~budget_s
    probe = max(20_000, min(seg, 200_000))
    r, dt = cpu_slice_run(pmin, nmin, nmax, probe)
    width = int(min(seg, max(probe, probe * budget_s / max(dt, 1e-3))))
    r, dt = cpu_slice_run(pmin, nmin, nmax, width)
    pairs = r["primecount"] * (nmax - nmin)
    return {"value": pairs / dt, "unit": "pair-steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"p in [{pmin}, {pmin + width}) of the workload ({r['primecount']} candidates, "
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
                         "sample": f"{args.steps} consecutive {width}-wide p-slices, oracle/oracle.c OpenMP "
                                   f"(the reference's OpenCL path has no runtime on this host)"},
        "e2e": {"value": value, "unit": "pair-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ GPU leg -----

def run_ours(args):
    import torch
    import factsieve_gb300 as fs
    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    dist = init_dist(ws, "nccl" if ws > 1 else None)
    wl = args.workload
    pmin, pmax, nmin, nmax, seg = WORKLOADS[wl]
    W = nmax - nmin
    nseg = (pmax - pmin + seg - 1) // seg

    def seg_range(i):
        lo = pmin + (i % nseg) * seg
        return lo, min(lo + seg, pmax)

    ctx = fs.Context(dev)
    stream = torch.cuda.Stream(device=dev)
    ctx.set_stream(stream.cuda_stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2

    # my segments: round-robin over ranks, K timed after W warm-up
    mine = [rank + ws * j for j in range(args.warmup + args.steps)]
    ctx.begin(pmin, pmax, nmin, nmax)
    with torch.cuda.stream(stream):
        for i in mine[: args.warmup]:
            ctx.segment(*seg_range(i))
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
            for j, i in enumerate(mine[args.warmup:]):
                ctx.segment(*seg_range(i))
                if j + 1 < args.steps:
                    flush.fill_(j & 0xFF)  # L2 flush between timed steps
            e1.record(stream)
        torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1)
    st = ctx.stats()
    ctx.set_timing(False)
    hits, raw, primecount, flags, rc = ctx.collect(cap)
    assert rc == 0, f"device flagged {flags}"
    pairs = primecount * W
    # max time over ranks, total work over ranks
    if dist:
        t = torch.tensor([ms, float(pairs), st["sieve_ms"], float(st["sieve_launches"]), float(primecount)],
                         dtype=torch.float64, device=dev)
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = t.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        ms, pairs = tmax[0].item(), tsum[1].item()
        primecount = int(tsum[4].item())
    value = pairs / (ms * 1e-3)

    # roofline of the dominant kernel, from this rank's events
    setup_prod = reference_setup_products(nmin)
    my_pc = primecount if not dist else int(t[4].item())
    products = my_pc * (W + setup_prod + 1)
    sieve_s = st["sieve_ms"] * 1e-3
    achieved = products / sieve_s / 1e9 if sieve_s > 0 else 0.0
    imad_ops, _ = ctx.bench_int_pipe(0, 20000)
    peak = imad_ops / IMAD_PER_PRODUCT / 1e9
    roof = {"bound": "imad", "achieved": achieved, "peak": peak, "unit": "Gmulmod/s",
            "frac": achieved / peak if peak else None, "traffic": None,
            "kernel": "sieve_kernel (setup+iterate+check, fused)",
            "kernel_ms_per_launch": st["sieve_ms"] / max(st["sieve_launches"], 1),
            "products_per_launch": products / max(st["sieve_launches"], 1),
            "peak_source": "measured IMAD stream on this GPU (fs_bench_int_pipe) / 20 IMAD per "
                           "reference Montgomery product",
            "share_of_step": (st["sieve_ms"] + 0.0) / ms if ms else None}

    # e2e through the public API with host buffers, on rank 0's first segments
    e2e = None
    if rank == 0:
        e2e_steps = max(1, min(args.steps, 3))
        ctx.set_stream(None)
        t0 = time.perf_counter()
        e2e_pairs = 0
        h2d = d2h = 0
        for i in range(e2e_steps):
            lo, hi = seg_range(i)
            r = ctx.sieve(lo, hi, nmin, nmax, threads=os.cpu_count() or 2)
            e2e_pairs += r.primecount * W
            words, layers, _ = fs.setup_plan(nmin)
            h2d += words.nbytes + layers.nbytes + 64
            d2h += 32 + 16 * r.nhits
        dt = time.perf_counter() - t0
        e2e = {"value": e2e_pairs / dt, "unit": "pair-steps/s", "h2d_bytes_per_step": h2d // e2e_steps,
               "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps,
               "path": "Context.sieve (fs_search_begin/segment/collect + fs_postprocess)"}

    if rank == 0:
        cpu = cpu_baseline(wl) if (ws == 1 and not args.no_cpu) else None
        line = {
            "metric": "(p,n) pair-steps/sec", "value": value, "unit": "pair-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (integer ranges; no dataset)",
            "config": {"workload": f"{wl}: p in [{pmin}, {pmax}), n in [{nmin}, {nmax})",
                       "step": f"one p-segment of {seg} (segment i of {nseg}, dealt round-robin to ranks)",
                       "parallelism": f"p-segments over {ws} GPU(s), no collective",
                       "l2": "flushed between timed steps (256 MiB write)",
                       "candidates_timed": primecount, "pair_steps_timed": pairs},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(st["launches"]),
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
