"""Benchmark: Bellard terms/s at hex position 1e10, 192-bit integer mode, on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one full pass of the hot path for one position: all 7 series, k in
[0, d) plus the 20-term tails, summed into the 192-bit result. On one GPU that
is one persistent term kernel + one combine kernel; on N > 1 GPUs (torchrun)
the position is split into 8N balanced work-mode jobs (cbl_plan_jobs), each
rank runs its share, and the 48-hex job partials are merged by an exact
integer add (workmodeSum), so the metric is time to the position on N GPUs.
value = 7*d terms (tails excluded) per second of device time. The default
N = 1 line also reports the batched-positions workload (4096 positions,
one persistent launch), the 1e11 position with checkpointed passes and its
P-8 overlap, and the digits the 106-bit double-double mode keeps. The
reference arm (--impl reference) times the reference's CPU implementation of
the same path on the host cores.
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
def _cpu_sample(d: int, L: int, threads: int):
    """The oracle over 7 series x 16 chunks of L terms spread evenly over
    k in [0, d): (terms, seconds)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    n = 0
    for f in range(7):
        for j in range(16):
            k0 = (d * j) // 16
            O.sum_range(d, f, k0, min(d, k0 + L), 3, threads)
            n += min(d, k0 + L) - k0
    return n, time.perf_counter() - t0


def cpu_sample_size(d: int, target_s: float, threads: int = 0) -> int:
    """Chunk length L for a sample of about target_s, from a probe that runs at
    least 0.5 s."""
    L = 4096
    while True:
        n, t = _cpu_sample(d, L, threads)
        if t >= 0.5 or L >= d:
            break
        L = min(d, int(L * max(2.0, 0.6 / max(t, 1e-3))))
    return max(256, min(d, int(n / max(t, 1e-6) * target_s / (7 * 16))))


def cpu_sample_rate(needD: int, target_s: float, threads: int = 0, L: int = 0):
    """The oracle (CPU restatement of the reference's path) on a bounded,
    stratified sample of the workload: per series, 16 chunks spread evenly
    over k in [0, d), sized (unless L is given) so the sample takes about
    target_s. Returns (terms/s, sample description, cores, seconds timed,
    terms timed)."""
    from oracle import oracle as O
    O.build()
    d, _ = O.pos_to_d(needD)
    cores = threads or os.cpu_count() or 1
    L = L or cpu_sample_size(d, target_s, threads)
    n, t = _cpu_sample(d, L, threads)
    return (n / t, "7 series x 16 chunks of %d k spread over [0,d) at position %d (%d terms, %.1f s)"
            % (L, needD, n, t), cores, t, n)


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


def workload_config(d: int) -> dict:
    """The config both arms print (identical, so the two lines compare)."""
    return {"workload": "pi hex position 1e10: 7 series x d=%d terms + 20-term tails, 192-bit fixed point" % d,
            "position": POSITION, "d": d, "mode": "192-bit integer",
            "inputs": "none: k and m are generated arithmetically; GPU steps flush L2 (256 MiB write) between "
                      "steps"}


def reference_sample(needD: int, L: int, threads: int):
    """The reference's own kernels (oracle/_ref, compiled from its OpenCL
    sources as C++; precision 2, the 192-bit integer mode) on a stratified
    sample of the workload: per series, 8 k-ranges of L terms spread over
    [0, d). Returns (terms/s, seconds, terms, threads)."""
    from oracle.ref_harness import build as R
    r = R.run(needD, 2, threads=threads, sample=(L, 8))
    n = 56 * L
    return r["terms_per_s"], n / r["terms_per_s"], n, r.get("threads", threads)


def reference_arm(args):
    """Each step times a bounded sample of the 1e10 workload on all host
    cores; value = terms of the timed samples / their seconds. The full
    position's time is extrapolated from that rate and labelled so."""
    world, rank, _ = dist_init()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    from oracle.ref_harness import build as R
    d, _ = O.pos_to_d(POSITION)
    use_ref = R.runnable()
    if use_ref:
        # size the sample from a probe of at least 0.5 s
        L = 1 << 16
        while True:
            rate, t, n, cores = reference_sample(POSITION, L, threads)
            if t >= 0.5:
                break
            L *= 4
        L = max(1 << 16, int(rate * args.ref_seconds / 56))
        desc = ("reference kernels (precision 2) on 7 series x 8 chunks of %d k spread over [0,d) at position %d"
                % (L, POSITION))
    else:
        L = cpu_sample_size(d, args.ref_seconds, threads)
    step_s, step_terms = [], []
    for i in range(args.warmup + args.steps):
        if use_ref:
            rate, t, n, cores = reference_sample(POSITION, L, threads)
        else:
            rate, desc, cores, t, n = cpu_sample_rate(POSITION, args.ref_seconds, threads, L)
            desc += ("; the reference's OpenCL/HSP host cannot run here and its kernels were not compiled for "
                     "this machine, so its CPU restatement (oracle/, Montgomery + exact long division) is timed")
        if i >= args.warmup:
            step_s.append(t)
            step_terms.append(n)
    timed_s, terms_timed = sum(step_s), sum(step_terms)
    value = terms_timed / timed_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * timed_s / len(step_s),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u32/u64 int",
        "data": "synthetic", "config": workload_config(d),
        "extrapolated": True, "timed_s": timed_s, "terms_timed": terms_timed,
        "ms_per_position_extrapolated": 7 * d / value * 1000.0,
        "step": "one bounded sample of the 1e10 workload (%d terms); the full position (%d terms) is "
                "extrapolated from the sampled rate" % (terms_timed // len(step_s), 7 * d),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference" if use_ref else "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def golden(name: str) -> dict:
    """A committed oracle fixture (tests/golden), or {} when absent."""
    path = os.path.join(ROOT, "tests", "golden", name)
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def agreeing_digits(a: str, b: str) -> int:
    n = 0
    for x, y in zip(a, b):
        if x != y:
            break
        n += 1
    return n


def ours_arm(args):
    world, rank, local = dist_init()
    if world > 1 or args.split:
        return split_arm(args, world, rank, local)
    import torch
    import clbellard_gb300 as C
    torch.cuda.set_device(local)
    C.load()
    needD = POSITION
    d, _ = C.pos_to_d(needD)
    ctx = C.Context(local, 1)
    if args.tile:
        ctx.set_tuning(args.tile, args.ctas)
    ctx.prepare([needD])
    info = ctx.prepared_info()
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")   # > 129 MB L2
    for _ in range(args.warmup):
        ctx.run_prepared()
    ctx.wait()
    result = "%048x" % ctx.read_results()[0]
    # peak: measured multiply-half issue rate of this GPU
    peak_ops, _ = ctx.probe_imad(4096)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    kern_ms = []
    n0 = ctx.launch_count
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
    launches = ctx.launch_count - n0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = sum(step_ms) / len(step_ms)
    terms = 7 * d
    value = terms / (ms / 1000.0)
    # end to end through the public call with host buffers (segment table
    # up, 24-byte result down, synchronised), same metric
    e2e_ms = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h = ctx.compute(needD)
        e2e_ms.append((time.perf_counter() - t0) * 1000.0)
    e2e_ms = sum(e2e_ms) / len(e2e_ms)
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
    exact = golden("oracle_big.json").get(str(needD), {})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "u32 int (192-bit fixed point)", "data": "synthetic",
        "config": workload_config(d),
        "launch": {"tile_terms": args.tile or 2048, "grid": info["grid"], "tiles": info["tiles"],
                   "segments": info["segments"]},
        "e2e": {"value": terms / (e2e_ms / 1000.0), "unit": UNIT,
                "h2d_bytes_per_step": 48 * info["segments"] + 4, "d2h_bytes_per_step": 24},
        "roofline": {"bound": "int", "achieved": achieved, "peak": peak_ops / 1e9, "unit": "Gmul/s",
                     "frac": achieved / (peak_ops / 1e9), "traffic": traffic,
                     "kernel": "terms192_kernel", "kernel_ms": kms,
                     "work": "32-bit multiply halves: 4S+12 per term (m<2^32), 18S+33 (m>=2^32)",
                     "peak_source": "measured mad.lo.u32 issue rate (dependent chains, one half each) on this "
                                    "GPU (no integer peak in MEASURED_PEAKS.json)"},
        "gpu_launches": launches,
        "result_hex": result,
        "result_equals_oracle": (result == exact["hex192"]) if exact else None,
        "clocks": clk.summary(),
    }
    ref = golden("ref_outputs.json").get(str(needD), {})
    if "mode2" in ref:
        # the reference's own 192-bit output at this position (its kernels run in full on a CPU)
        line["digits_equal_to_reference_192bit"] = agreeing_digits(result, ref["mode2"])
    pipe = issue_fraction(kms)
    if pipe:
        line["roofline"]["pipe"] = pipe
    if h != result:
        line["error"] = "e2e result differs from device-timed result"
    if not args.no_cpu_baseline:
        r, desc, cores, _, _ = cpu_sample_rate(needD, args.cpu_seconds)
        line["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    if args.dd:
        line["dd_compare"] = dd_compare(C, local, needD, d)
        line["dd_digits_kept"] = dd_digits(C, local, needD, result, exact)
    ctx.close()
    if args.extras:
        line["batch"] = batch_report(C, local, args)
        line["large"] = large_report(C, local, args)
    print(json.dumps(line), flush=True)
    return 0


def issue_fraction(kernel_ms: float):
    """The FMA-heavy pipe (integer multiplies) of the term kernel at 1e10
    from a committed one-pass ncu capture of the same workload
    (profiles/terms192_issue.json): its busy fraction as ncu reports it, and
    its warp-instruction issue rate against one warp instruction per 2 cycles
    per SM sub-partition, with this run's kernel time at the profile's clock.
    Wide and high multiplies hold the pipe for two issue cycles, so the busy
    fraction is the higher of the two."""
    path = os.path.join(ROOT, "profiles", "terms192_issue.json")
    try:
        with open(path) as f:
            p = json.load(f)
    except (OSError, ValueError):
        return None
    peak = p["sms"] * p["smsp_per_sm"] * p["warp_inst_per_cycle_per_smsp"] * p["sm_mhz"] * 1e6
    rate = p["fmaheavy_warp_inst_per_launch"] / (kernel_ms / 1000.0)
    return {"fmaheavy_pipe_busy_ncu": p["fmaheavy_pipe_busy_pct"] / 100.0,
            "fmaheavy_warp_inst_per_launch": p["fmaheavy_warp_inst_per_launch"],
            "fmaheavy_issue_frac": rate / peak, "source": p.get("source", path)}


def split_arm(args, world, rank, local):
    """One position sharded over ranks: 8 balanced jobs per rank
    (cbl_plan_jobs), each run through cbl_run_job_range, merged with the
    exact 48-hex add (workmode.distributed_sum) -- the reference's work mode
    (Bellard_192.hsp:298-340, workmodeSum0_6.hsp:10-31) done in-process."""
    import torch
    import clbellard_gb300 as C
    from clbellard_gb300 import workmode
    torch.cuda.set_device(local)
    C.load()
    needD = POSITION
    d, _ = C.pos_to_d(needD)
    ctx = C.Context(local, 1)
    stream = torch.cuda.ExternalStream(ctx.stream, device=local)
    run = lambda s, k0, k1: ctx.run_job_range(needD, s, k0, k1)   # noqa: E731
    for _ in range(args.warmup):
        split_position(needD, world, rank, run)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    wall = []
    n0 = ctx.launch_count
    merged = None
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            barrier(world)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ev[i][0].record(stream)
            mine = split_position(needD, world, rank, run, merge=False)
            ev[i][1].record(stream)
            torch.cuda.synchronize()
            merged = workmode.distributed_sum(mine) if world > 1 else C.workmode_sum(mine)
            wall.append(time.perf_counter() - t0)
    launches = ctx.launch_count - n0
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev) / args.steps, world)
    e2e_s = max_over_ranks(sum(wall) / len(wall), world)
    exact = golden("oracle_big.json").get(str(needD), {})
    line = {
        "metric": METRIC, "value": 7 * d / (ms / 1000.0), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "u32 int (192-bit fixed point)", "data": "synthetic",
        "config": workload_config(d),
        "launch": {"split": "%d balanced jobs (cbl_plan_jobs), %d per rank, merged by an exact 48-hex add"
                            % (8 * world, 8)},
        "e2e": {"value": 7 * d / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 48 * 7 * 8,
                "d2h_bytes_per_step": 24 * 8,
                "note": "host wall time including the job partials' merge; h2d is the bound of 8 jobs' segment "
                        "tables (48 B per segment, at most 7 per job), d2h the 8 partials"},
        "gpu_launches": launches,
        "result_hex": merged,
        "result_equals_oracle": (merged == exact["hex192"]) if exact else None,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def split_position(needD, world, rank, run_range, merge=True, jobs_per_rank=8):
    """This rank's share of the balanced plan for needD: run_range(s, k0, k1)
    gives each job's 48-hex partial. With merge, all ranks' partials are
    summed (workmode.distributed_sum when world > 1) and the merged hex is
    returned; otherwise this rank's partials."""
    import clbellard_gb300 as C
    from clbellard_gb300 import workmode
    jobs = C.plan_jobs(needD, max(7, jobs_per_rank * world))
    mine = [run_range(s, k0, k1) for s, k0, k1 in workmode.shard(jobs, rank, world)]
    if not merge:
        return mine
    return workmode.distributed_sum(mine) if world > 1 else C.workmode_sum(mine)


def batch_positions(n: int, seed: int = 4096):
    """n reference positions drawn log-uniform in [1e3, 1e9] (numpy
    default_rng(seed)), rounded to integers."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [int(x) for x in np.rint(10.0 ** rng.uniform(3.0, 9.0, size=n))]


def batch_report(C, device, args, steps=2, warmup=1, tune_n=64):
    """Batched positions (4096 log-uniform in [1e3, 1e9]) in one persistent
    pass (graph replay), autotuned on a subsample, against the single-position
    rate at 1e9 with the same tuning; every position <= 1e5 is checked against
    the oracle and the 8 largest against single-position compute."""
    import torch
    pos = batch_positions(args.npos)
    ds = [C.pos_to_d(p)[0] for p in pos]
    terms = 7 * sum(ds)
    ctx = C.Context(device, 1)
    tile, ctas, tune_ms = ctx.autotune(pos[:tune_n], force=True)
    ctx.prepare(pos)
    info = ctx.prepared_info()
    for _ in range(warmup):
        ctx.run_prepared()
    ctx.wait()
    ms = []
    n0 = ctx.launch_count
    with ClockSampler(device) as clk:
        for _ in range(steps):
            ctx.run_prepared()
            ms.append(ctx.kernel_ms())
    launches = ctx.launch_count - n0
    res = ctx.read_results()
    kms = sum(ms) / len(ms)
    ctx.prepare([10 ** 9])
    ctx.run_prepared()
    ctx.run_prepared()
    single_ms = ctx.kernel_ms()
    single_rate = 7 * C.pos_to_d(10 ** 9)[0] / (single_ms / 1000.0)
    t0 = time.perf_counter()
    res2 = ctx.batch(pos)
    e2e_s = time.perf_counter() - t0
    # parity of a seeded subset
    from oracle import oracle as O
    small = [i for i, p in enumerate(pos) if p <= 10 ** 5]
    oracle_ok = all(res[i] == O.result(ds[i], 0, 3) for i in small)
    largest = sorted(range(len(pos)), key=lambda i: -pos[i])[:8]
    single_ok = all("%048x" % res[i] == ctx.compute(pos[i]) for i in largest)
    ctx.close()
    torch.cuda.synchronize()
    value = terms / (kms / 1000.0)
    return {"value": value, "unit": UNIT, "ms_per_pass": kms, "steps": steps, "warmup": warmup,
            "workload": "%d positions log-uniform in [1e3, 1e9] (numpy default_rng(4096)), 192-bit, one "
                        "persistent launch per pass (CUDA graph replay)" % args.npos,
            "terms": terms, "segments": info["segments"], "tiles": info["tiles"], "tile_terms": tile,
            "ctas_per_sm": ctas, "autotune": "forced sweep on the first %d positions (%.1f ms best)"
                                              % (tune_n, tune_ms),
            "single_position_1e9_terms_per_s": single_rate, "sweep_over_single": value / single_rate,
            "e2e": {"value": terms / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 48 * info["segments"] + 4 * len(pos),
                    "d2h_bytes_per_step": 24 * len(pos)},
            "gpu_launches": launches, "clocks": clk.summary(),
            "results_consistent": res == res2,
            "checked": {"positions_le_1e5_vs_oracle": len(small), "oracle_ok": oracle_ok,
                        "largest_8_vs_single_compute": single_ok}}


def large_report(C, device, args, needD=10 ** 11):
    """Position 1e11 in 192-bit mode, run as time-budgeted passes with a
    checkpoint saved and restored between them; hex position P-8 overlap;
    the 106-bit double-double mode at the same position and the digits it
    keeps against the 192-bit result (and the exact value when committed)."""
    import torch
    d, _ = C.pos_to_d(needD)
    out = {"position": needD, "d": d}
    with C.Context(device, 1) as ctx:
        ctx.prepare([needD])
        t0 = time.perf_counter()
        passes, done, total = 0, 0, 1
        while done < total:
            done, total = ctx.run_prepared_budget(args.large_slice_ms)
            passes += 1
            if done < total:
                blob = ctx.checkpoint()
                ctx.restore(blob)
        h192 = "%048x" % ctx.read_results()[0]
        out["ms_192"] = (time.perf_counter() - t0) * 1000.0
        out["budgeted_passes"] = passes
        out["terms_per_s_192"] = 7 * d / (out["ms_192"] / 1000.0)
        out["hex192"] = h192
        exact = golden("oracle_big.json").get(str(needD), {})
        if exact:
            out["equals_oracle_192"] = h192 == exact["hex192"]
            out["digits_vs_exact_256"] = agreeing_digits(h192, exact["hex256"])
        # the result's first digit is hex position (10d + 6)/4 + 1; the value
        # at hex position P - 8 must repeat it from its ninth digit on
        p = (10 * d + 6) // 4 + 1
        hm8 = ctx.compute_hexpos(p - 8)
        out["hexpos"] = p
        out["overlap_digits_p_minus_8"] = agreeing_digits(hm8[8:], h192)
    with C.Context(device, 0) as ctxdd:
        t0 = time.perf_counter()
        hdd = ctxdd.compute(needD)
        out["ms_dd"] = (time.perf_counter() - t0) * 1000.0
        out["hex_dd"] = hdd
        out["dd_digits_vs_192"] = agreeing_digits(hdd, h192)
        if exact:
            out["dd_digits_vs_exact_256"] = agreeing_digits(hdd, exact["hex256"])
    torch.cuda.synchronize()
    return out


def dd_digits(C, device, needD, h192, exact):
    """The 106-bit double-double mode at the same position: hex digits that
    agree with the 192-bit result and with the exact 256-bit value."""
    with C.Context(device, 0) as ctxdd:
        t0 = time.perf_counter()
        hdd = ctxdd.compute(needD)
        ms = (time.perf_counter() - t0) * 1000.0
    r = {"position": needD, "hex_dd": hdd, "ms_dd": ms, "digits_vs_192": agreeing_digits(hdd, h192)}
    ref = golden("ref_outputs.json").get(str(needD), {})
    if "mode0" in ref:
        r["digits_vs_reference_mode0"] = agreeing_digits(hdd, ref["mode0"])
    if exact:
        r["digits_vs_exact_256"] = agreeing_digits(hdd, exact["hex256"])
        r["digits_192_vs_exact_256"] = agreeing_digits(h192, exact["hex256"])
    return r


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


def batch_arm(args):
    """The batched-positions workload alone, as its own line."""
    import clbellard_gb300 as C
    import torch
    torch.cuda.set_device(0)
    C.load()
    r = batch_report(C, 0, args, steps=args.steps, warmup=args.warmup, tune_n=256)
    line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_pass"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32 int (192-bit fixed point)", "data": "synthetic",
            "config": {"workload": r["workload"]}, "e2e": r["e2e"], "gpu_launches": r["gpu_launches"],
            "clocks": r["clocks"], "batch": r}
    print(json.dumps(line), flush=True)
    return 0


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
    ap.add_argument("--split", action="store_true", help="shard the position into jobs even on one GPU")
    ap.add_argument("--dd", action="store_true", default=True)
    ap.add_argument("--no-dd", dest="dd", action="store_false")
    ap.add_argument("--extras", action="store_true", default=True,
                    help="also report the batched-positions and 1e11 workloads (default)")
    ap.add_argument("--no-extras", dest="extras", action="store_false")
    ap.add_argument("--large-slice-ms", type=float, default=3000.0)
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
