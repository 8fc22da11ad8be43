"""Work mode: worklist files, per-job result files, and sharding jobs over
processes / GPUs (Bellard_192.hsp:176-246, 298-348, 514-533; workmodeSum0_6.hsp).

A job is (s, b): series s, k in [b*BATCHSIZE, (b+1)*BATCHSIZE). Each job's
numer-weighted 192-bit partial is written as 48 hex digits in
<workdir>/<s>/<s>_<b>.txt; the answer is their sum mod 16^48. The merge is an
exact integer add, so any assignment of jobs to processes gives the same bits.
"""
from __future__ import annotations

import os
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Tuple

from . import BATCHSIZE, Context, load, workmode_sum

MAX_DIGITS = 999999999999999999


@dataclass
class Worklist:
    digits: int
    precision: int
    jobs: List[Tuple[int, int]] = field(default_factory=list)
    # explicit k-ranges of balanced jobs: (s, b) -> (k0, k1); jobs without an
    # entry cover the reference's batch [b * BATCHSIZE, (b + 1) * BATCHSIZE)
    ranges: dict = field(default_factory=dict)


def parse_worklist(text: str) -> Worklist:
    """Line 0 'digits=N', line 1 'precision=P ...', then 's_b' lines
    (Bellard_192.hsp:176-189, 229-246)."""
    lines = text.replace("\r\n", "\n").replace("\r", "\n").split("\n")
    if len(lines) < 2:
        raise ValueError("worklist needs a digits line and a precision line")
    dstr = lines[0].replace("digits", "").replace("=", "").replace(" ", "")
    digits_raw = "".join(ch for ch in dstr if ch.isdigit())
    digits = min(max(int(digits_raw) if digits_raw else 0, 0), MAX_DIGITS)
    pstr = lines[1].replace("precision", "").replace("=", "").replace(" ", "")
    precision = int(pstr[0]) if pstr[:1] in ("0", "1", "2") else -1
    if not (5 <= digits <= MAX_DIGITS) or precision < 0:
        raise ValueError("invalid worklist header (digits=%r precision=%r)" % (lines[0], lines[1]))
    jobs, ranges = [], {}
    for ln in lines[2:]:
        parts = ln.split()
        if not parts:
            continue
        tok = parts[0]
        if len(tok) >= 3 and tok[0].isdigit() and tok[1] == "_" and tok[2:].isdigit():
            job = (int(tok[0]), int(tok[2:]))
            jobs.append(job)
            # extension: "s_b k0 k1" gives the job an explicit k-range
            if len(parts) >= 3 and parts[1].isdigit() and parts[2].isdigit():
                ranges[job] = (int(parts[1]), int(parts[2]))
    return Worklist(digits, precision, jobs, ranges)


def format_worklist(wl: Worklist) -> str:
    out = ["digits=%d" % wl.digits, "precision=%d (0=106bit , 1=192bit)" % wl.precision]
    for j in wl.jobs:
        out.append("%d_%d %d %d" % (j + wl.ranges[j]) if j in wl.ranges else "%d_%d" % j)
    return "\n".join(out) + "\n"


def balanced_worklist(needD: int, njobs: int, precision: int = 1) -> Worklist:
    """njobs jobs of about equal device time (cbl_plan_jobs), numbered per series."""
    from . import plan_jobs
    wl = Worklist(needD, precision)
    count = [0] * 7
    for s, k0, k1 in plan_jobs(needD, njobs):
        job = (s, count[s])
        count[s] += 1
        wl.jobs.append(job)
        wl.ranges[job] = (k0, k1)
    return wl


def all_jobs(d: int, batchsize: int = BATCHSIZE) -> List[Tuple[int, int]]:
    """Every job needed for position d: (s, b) for b = 0 .. d // batchsize."""
    return [(s, b) for s in range(7) for b in range(d // batchsize + 1)]


def shard(jobs: Sequence[Tuple[int, int]], rank: int, world: int) -> List[Tuple[int, int]]:
    """Round-robin assignment of jobs to ranks (disjoint, covering)."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    return [j for i, j in enumerate(jobs) if i % world == rank]


def job_path(workdir: str, s: int, b: int) -> str:
    return os.path.join(workdir, str(s), "%d_%d.txt" % (s, b))


def write_job(workdir: str, s: int, b: int, hex48: str, deviceno: int, devname: str, ms: int):
    load()
    from . import _lib, _check
    _check(_lib.cbl_job_write(workdir.encode(), s, b, hex48.encode(), deviceno, devname.encode(), int(ms)),
           "cbl_job_write")


def read_job(workdir: str, s: int, b: int) -> Optional[str]:
    import ctypes
    load()
    from . import _lib
    out = ctypes.create_string_buffer(49)
    rc = _lib.cbl_job_read(workdir.encode(), s, b, out)
    return out.value.decode() if rc == 0 else None


def workdir_sum(workdir: str):
    """workmodeSum0_6: (hex48, files per series)."""
    import ctypes
    load()
    from . import _lib, _check
    out = ctypes.create_string_buffer(49)
    counts = (ctypes.c_int * 7)()
    _check(_lib.cbl_workdir_sum(workdir.encode(), out, counts), "cbl_workdir_sum")
    return out.value.decode(), list(counts)


JobFn = Callable[[int, int, int, int], Optional[str]]   # (needD, s, b, batchsize) -> hex48 | None
RangeFn = Callable[[int, int, int, int], Optional[str]]  # (needD, s, k0, k1) -> hex48 | None


def run_jobs(jobs, needD: int, workdir: str, job_fn: JobFn, batchsize: int = BATCHSIZE, deviceno: int = 0,
             devname: str = "", ranges: Optional[dict] = None, range_fn: Optional[RangeFn] = None) -> int:
    """*Batchloop (Bellard_192.hsp:298-340): run each job not already on disk,
    write its file. Jobs listed in `ranges` run over their explicit k-range
    with range_fn. Returns the number of jobs run."""
    n = 0
    for s, b in jobs:
        if read_job(workdir, s, b) is not None:       # finished earlier (:307-308)
            continue
        t0 = time.time()
        if ranges and (s, b) in ranges:
            h = range_fn(needD, s, *ranges[(s, b)])
        else:
            h = job_fn(needD, s, b, batchsize)
        if h is None:                                 # k_start > d (:306)
            continue
        write_job(workdir, s, b, h, deviceno, devname, int((time.time() - t0) * 1000))
        n += 1
    return n


def gpu_job_fn(ctx: Context) -> JobFn:
    return lambda needD, s, b, bs: ctx.run_job(needD, s, b, bs)


def gpu_range_fn(ctx: Context) -> RangeFn:
    return lambda needD, s, k0, k1: ctx.run_job_range(needD, s, k0, k1)


def merge_gathered(parts: Sequence[Sequence[str]]) -> str:
    """Merge the per-rank lists of job partials (the only exchange step)."""
    flat = [h for p in parts for h in p]
    return workmode_sum(flat)


def distributed_sum(my_partials: Sequence[str]) -> str:
    """All ranks contribute their job partials; every rank gets the merged sum.
    Uses torch.distributed (gloo on CPU, nccl on GPUs) all_gather_object:
    48 hex characters per job, nothing else crosses ranks."""
    import torch.distributed as dist
    world = dist.get_world_size()
    gathered = [None] * world
    dist.all_gather_object(gathered, list(my_partials))
    return merge_gathered(gathered)
