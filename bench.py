"""Benchmark: Bellard terms/s at hex position 1e10, 192-bit integer mode, on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full pass of the hot path for one position: all 7 series, k in
[0, d) plus the 20-term tails, summed into the 192-bit result (one persistent
term kernel + one combine kernel). value = 7*d terms (tails excluded) per
second of device time, summed over ranks (weak scaling: rank r computes
position 1e10 + 10r). The reference arm (--impl reference) times the
reference's CPU implementation of the same path on the host cores.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

POSITION = 10 ** 10
METRIC = "Bellard terms/s"
UNIT = "terms/s"


# ------------------------------------------------------------ work model --
def algorithmic_mults(d: int) -> int:
    """Algorithmic 32-bit multiply halves of one position (tails excluded):
    per term W = 4S + 12 for m < 2^32 and 18S + 33 for m >= 2^32, with
    S = bitlen(10(d-k)) - 1 squarings (the fixed work definition used for the
    roofline)."""
    from clbellard_gb300 import formula
    total = 0
    for f in range(7):
        _, _, den0, den1 = formula(f)
        k32 = max(0, ((1 << 32) - den1 + den0 - 1) // den0)   # first k with m >= 2^32
        # e = d - k in [1, d]; S = bitlen(10e) - 1; split e by bitlen of 10e
        for b in range(1, 70):
            lo_e = max(1, -(-(1 << (b - 1)) // 10))          # smallest e with 10e >= 2^(b-1)
            hi_e = min(d, ((1 << b) - 1) // 10)              # largest e with 10e < 2^b
            if hi_e < lo_e:
                continue
            S = b - 1
            # k = d - e, so e in [lo_e, hi_e] <-> k in [d - hi_e, d - lo_e]
            ka, kb = d - hi_e, d - lo_e
            n32 = max(0, min(kb, k32 - 1) - ka + 1)           # k < k32: m < 2^32
            n64 = (kb - ka + 1) - n32
            total += n32 * (4 * S + 12) + n64 * (18 * S + 33)
    return total


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline --
def cpu_sample_rate(needD: int, target_s: float, threads: int = 0):
    """The oracle (CPU restatement of the reference's path) on a bounded,
    stratified sample of the workload: per series, 16 chunks spread evenly
    over k in [0, d). Returns (terms/s, sample description, cores)."""
    from oracle import oracle as O
    O.build()
    d, _ = O.pos_to_d(needD)
    cores = threads or os.cpu_count() or 1

    def run(L):
        t0 = time.perf_counter()
        n = 0
        for f in range(7):
            for j in range(16):
                k0 = (d * j) // 16
                O.sum_range(d, f, k0, min(d, k0 + L), 3, threads)
                n += min(d, k0 + L) - k0
        return n, time.perf_counter() - t0

    n, t = run(256)
    rate = n / max(t, 1e-6)
    L = max(256, int(rate * target_s / (7 * 16)))
    n, t = run(L)
    return n / t, "7 series x 16 chunks of %d k spread over [0,d) at position %d (%d terms)" % (L, needD, n), cores


# ----------------------------------------------------------------- arms --
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except ImportError:
            backend = "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reference_sample_rate(needD: int, target_s: float, threads: int):
    """The reference's own kernels (oracle/_ref, compiled from its OpenCL
    sources as C++; precision 2, the 192-bit integer mode) on a stratified
    sample of the workload: per series, 8 k-ranges spread over [0, d)."""
    from oracle.ref_harness import build as R
    r = R.run(needD, 2, threads=threads, sample=(1 << 19, 8))
    rate = r["terms_per_s"]
    L = max(1 << 19, int(rate * target_s / 56))
    r = R.run(needD, 2, threads=threads, sample=(L, 8))
    return r["terms_per_s"], ("reference kernels (precision 2) on 7 series x 8 chunks of %d k spread over [0,d) "
                              "at position %d" % (L, needD)), r.get("threads", threads)


def reference_arm(args):
    world, rank, _ = dist_init()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    from oracle.ref_harness import build as R
    d, _ = O.pos_to_d(POSITION)
    use_ref = R.runnable()
    rates = []
    desc = ""
    cores = threads
    for i in range(args.warmup + args.steps):
        if use_ref:
            r, desc, cores = reference_sample_rate(POSITION, args.ref_seconds, threads)
        else:
            r, desc, cores = cpu_sample_rate(POSITION, args.ref_seconds, threads)
            desc += ("; the reference's OpenCL/HSP host cannot run here and its kernels were not compiled for "
                     "this machine, so its CPU restatement (oracle/, Montgomery + exact long division) is timed")
        if i >= args.warmup:
            rates.append(r)
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 7 * d / value * 1000.0,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32/u64 int", "data": "synthetic",
        "config": {"workload": "pi hex position 1e10, 192-bit fixed point, 7 series x d=%d terms" % d,
                   "position": POSITION, "d": d, "mode": "192-bit"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference" if use_ref else "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ours_arm(args):
    world, rank, local = dist_init()
    import torch
    import clbellard_gb300 as C
    torch.cuda.set_device(local)
    C.load()
    needD = POSITION + 10 * rank
    d, _ = C.pos_to_d(needD)
    ctx = C.Context(local, 1)
    if args.tile:
        ctx.set_tuning(args.tile, args.ctas)
    ctx.prepare([needD])
    info = ctx.prepared_info()
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2
    # warm-up (also checks the result against the published digits)
    for _ in range(args.warmup):
        ctx.run_prepared()
    ctx.wait()
    result = "%048x" % ctx.read_results()[0]
    # peak: measured multiply-half issue rate of this GPU
    peak_ops, _ = ctx.probe_imad(4096)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kern_ms = []
    n0 = ctx.launch_count
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(i & 0xff)                  # L2 flush, outside the timed interval
            ev[i][0].record(stream)
            ctx.run_prepared()
            ev[i][1].record(stream)
            kern_ms.append(ctx.kernel_ms())
        torch.cuda.synchronize()
    barrier(world)
    launches = ctx.launch_count - n0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(sum(step_ms) / len(step_ms), world)
    terms = 7 * d
    value = terms * world / (ms / 1000.0)
    # end to end through the public call with host buffers (segment table
    # up, 24-byte result down, synchronised), same metric
    e2e_ms = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = ctx.compute(needD)
        e2e_ms.append((time.perf_counter() - t0) * 1000.0)
    e2e_ms = max_over_ranks(sum(e2e_ms) / len(e2e_ms), world)
    kms = sum(kern_ms) / len(kern_ms)
    mults = algorithmic_mults(d)
    achieved = mults / (kms / 1000.0) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "terms192_traffic.json")
    if os.path.exists(tp):
        try:
            traffic = json.load(open(tp)).get("bytes_per_launch")
        except (OSError, ValueError):
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32 int (192-bit fixed point)", "data": "synthetic",
        "config": {"workload": "pi hex position 1e10, 192-bit fixed point, 7 series x d=%d terms + 20-term tails"
                               % d, "position": needD, "d": d, "mode": "192-bit integer",
                   "l2": "flushed between steps (256 MiB write); the path reads no HBM inputs",
                   "tile_terms": args.tile or 2048, "grid": info["grid"], "tiles": info["tiles"]},
        "e2e": {"value": terms * world / (e2e_ms / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": 48 * info["segments"] + 4, "d2h_bytes_per_step": 24},
        "roofline": {"bound": "int", "achieved": achieved, "peak": peak_ops / 1e9, "unit": "Gmul/s",
                     "frac": achieved / (peak_ops / 1e9), "traffic": traffic,
                     "kernel": "terms192_kernel", "kernel_ms": kms,
                     "work": "32-bit multiply halves: 4S+12 per term (m<2^32), 18S+33 (m>=2^32)",
                     "peak_source": "measured mad.lo.u32 issue rate (dependent chains, one half each) on this "
                                    "GPU (no integer peak in MEASURED_PEAKS.json)"},
        "gpu_launches": launches,
        "result_hex": result,
        "clocks": clk.summary(),
    }
    if h != result:
        line["error"] = "e2e result differs from device-timed result"
    if rank == 0 and not args.no_cpu_baseline:
        r, desc, cores = cpu_sample_rate(needD, args.cpu_seconds)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    if rank == 0 and args.dd:
        line["dd_compare"] = dd_compare(C, local, needD, d)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def batch_positions(n: int, seed: int = 4096):
    """n reference positions drawn log-uniform in [1e3, 1e9] (numpy
    default_rng(seed)), rounded to integers."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [int(x) for x in np.rint(10.0 ** rng.uniform(3.0, 9.0, size=n))]


def batch_arm(args):
    """Batched positions: one persistent pass over all positions (graph
    replay), autotuned on a subsample; reported against the single-position
    rate at 1e9 with the same tuning."""
    import torch
    import clbellard_gb300 as C
    torch.cuda.set_device(0)
    pos = batch_positions(args.npos)
    ds = [C.pos_to_d(p)[0] for p in pos]
    terms = 7 * sum(ds)
    ctx = C.Context(0, 1)
    tile, ctas, tune_ms = ctx.autotune(pos[:256], force=True)
    ctx.prepare(pos)
    info = ctx.prepared_info()
    for _ in range(args.warmup):
        ctx.run_prepared()
    ctx.wait()
    ms = []
    n0 = ctx.launch_count
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            ctx.run_prepared()
            ms.append(ctx.kernel_ms())
    launches = ctx.launch_count - n0
    res = ctx.read_results()
    kms = sum(ms) / len(ms)
    # single position at the top of the range, same tuning
    ctx.prepare([10 ** 9])
    ctx.run_prepared()
    ctx.run_prepared()
    single_ms = ctx.kernel_ms()
    single_rate = 7 * C.pos_to_d(10 ** 9)[0] / (single_ms / 1000.0)
    # end to end: the public batch call with host arrays
    t0 = time.perf_counter()
    res2 = ctx.batch(pos)
    e2e_s = time.perf_counter() - t0
    value = terms / (kms / 1000.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": kms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32 int (192-bit fixed point)", "data": "synthetic",
        "config": {"workload": "%d positions log-uniform in [1e3, 1e9] (numpy default_rng(4096)), 192-bit, one "
                               "persistent launch per pass (CUDA graph replay)" % args.npos,
                   "positions": args.npos, "terms": terms, "segments": info["segments"], "tiles": info["tiles"],
                   "tile_terms": tile, "ctas_per_sm": ctas, "autotune_sample_ms": tune_ms},
        "single_position_1e9_terms_per_s": single_rate,
        "sweep_over_single": value / single_rate,
        "e2e": {"value": terms / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 48 * info["segments"] + 4 * args.npos,
                "d2h_bytes_per_step": 24 * args.npos},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "results_consistent": res == res2,
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def dd_compare(C, device, needD, d):
    """192-bit integer vs 106-bit double-double kernels on the same sample of
    the 1e10 workload: per series, 8 chunks of 2^24 k spread over [0, d),
    timed with CUDA events on each context's stream."""
    import torch
    L = 1 << 24
    chunks = [(f, (d * j) // 8) for f in range(7) for j in range(8)]
    out = {}
    for prec in (1, 0):
        ctx = C.Context(device, prec)
        stream = torch.cuda.ExternalStream(ctx.stream, device=device)
        for rep in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for f, k0 in chunks:
                _, sign, den0, den1 = C.formula(f)
                ctx.Set0mem()
                ctx.Sglobal64mtg(k0, d, min(d, k0 + L), sign, den0, den1)
            e1.record(stream)
            ctx.wait()
            dt = e0.elapsed_time(e1) / 1000.0
        out["dd" if prec == 0 else "int192"] = len(chunks) * L / dt
        ctx.close()
    out["ratio_int192_over_dd"] = out["int192"] / out["dd"]
    out["sample"] = "7 series x 8 chunks of 2^24 k at position %d, CUDA events" % needD
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--ctas", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=6.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", default="single", choices=["single", "batch"])
    ap.add_argument("--npos", type=int, default=4096)
    ap.add_argument("--dd", action="store_true", default=True)
    ap.add_argument("--no-dd", dest="dd", action="store_false")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    if args.config == "batch":
        return batch_arm(args)
    return ours_arm(args)


if __name__ == "__main__":
    sys.exit(main())
