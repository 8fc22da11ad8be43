"""Work-mode host logic on the CPU: worklist format, job files, the
workmodeSum merge, balanced plans, and sharding jobs over 2 gloo ranks. Job
partials come from the oracle here (the CPU stands in for the GPUs only in
these tests)."""
import os

import pytest

from conftest import load_golden
from workmode_helpers import oracle_job, oracle_range


def test_parse_sample_worklist():
    from clbellard_gb300 import workmode as W
    # the reference's work/worklist_sample.txt layout
    text = "digits=200000000\r\nprecision=1 (0=106bit , 1=192bit)\r\n0_0\r\n1_0\r\n2_0\r\n3_0\r\n4_0\r\n5_0\r\n6_0"
    wl = W.parse_worklist(text)
    assert wl.digits == 200000000 and wl.precision == 1
    assert wl.jobs == [(s, 0) for s in range(7)]
    assert W.parse_worklist(W.format_worklist(wl)).jobs == wl.jobs
    with pytest.raises(ValueError):
        W.parse_worklist("digits=3\nprecision=1\n")
    with pytest.raises(ValueError):
        W.parse_worklist("digits=1000\nprecision=x\n")


def test_job_files_roundtrip(tmp_path, cbl):
    from clbellard_gb300 import workmode as W
    h = "0123456789abcdef" * 3
    W.write_job(str(tmp_path), 3, 17, h, 0, "NVIDIA GB300", 1234)
    raw = open(os.path.join(tmp_path, "3", "3_17.txt"), "rb").read()
    assert raw == (h + "\r\n0\tNVIDIA GB300\r\n1234ms").encode()
    assert W.read_job(str(tmp_path), 3, 17) == h
    assert W.read_job(str(tmp_path), 3, 18) is None


def test_workdir_sum_equals_normal_mode(tmp_path, cbl, oracle):
    """Jobs with a small batch size, merged as workmodeSum does, give the
    normal-mode result bit for bit."""
    from clbellard_gb300 import workmode as W
    needD = 100000
    d, _ = oracle.pos_to_d(needD)
    bs = 7919
    jobs = W.all_jobs(d, bs)
    n = W.run_jobs(jobs, needD, str(tmp_path), oracle_job(oracle, bs), batchsize=bs)
    assert n == len(jobs)
    # a second pass finds every file and runs nothing (Bellard_192.hsp:307-308)
    assert W.run_jobs(jobs, needD, str(tmp_path), oracle_job(oracle, bs), batchsize=bs) == 0
    total, counts = W.workdir_sum(str(tmp_path))
    assert counts == [d // bs + 1] * 7
    assert total == oracle.to_hex(oracle.result(d, 0, 3), 3) == load_golden("oracle_small.json")["100000"]["hex192"]


def test_skip_past_d(cbl, oracle):
    fn = oracle_job(oracle, 1000)
    d, _ = oracle.pos_to_d(10000)
    assert fn(10000, 0, d // 1000 + 1, 1000) is None


@pytest.mark.parametrize("needD,njobs", [(10, 7), (10, 50), (100000, 16), (10 ** 10, 64), (10 ** 17, 200)])
def test_plan_tiles_each_series(cbl, oracle, needD, njobs):
    """Each series' ranges tile [0, d + 20) in order, only the last reaches d."""
    d, _ = oracle.pos_to_d(needD)
    plan = cbl.plan_jobs(needD, njobs)
    assert 7 <= len(plan) <= njobs
    for s in range(7):
        rs = [(k0, k1) for f, k0, k1 in plan if f == s]
        assert rs and rs[0][0] == 0 and rs[-1][1] == d + 20
        assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
        assert all(k0 < k1 for k0, k1 in rs)
        assert all(k1 < d for _, k1 in rs[:-1])
    with pytest.raises(cbl.CblError):
        cbl.plan_jobs(needD, 6)


def test_plan_balances_modelled_cost(cbl, oracle):
    """Per-term cost model (ladder bits + 8) x kind step cost, summed with
    numpy over every term: planned jobs are within 10% of each other."""
    import numpy as np
    needD = 10 ** 6
    d, _ = oracle.pos_to_d(needD)
    den = [(4, 1), (4, 3), (10, 1), (10, 3), (10, 5), (10, 7), (10, 9)]
    plan = cbl.plan_jobs(needD, 21)
    costs = []
    for s, k0, k1 in plan:
        k = np.arange(k0, min(k1, d), dtype=np.uint64)
        bits = np.floor(np.log2((10 * (d - k)).astype(np.float64))) + 1
        m = den[s][0] * k + den[s][1]
        step = np.where(m < 2 ** 28, 7.0, 9.0)             # m < 4e6 here: the two smallest kinds
        costs.append(float(((bits + 8) * step).sum()))
    assert max(costs) / min(costs) < 1.10


def test_balanced_worklist_sum_equals_normal_mode(tmp_path, cbl, oracle):
    """A balanced worklist written, parsed, run and merged gives the normal-mode bits."""
    from clbellard_gb300 import workmode as W
    needD = 100000
    wl = W.balanced_worklist(needD, 12)
    text = W.format_worklist(wl)
    assert all(len(ln.split()) == 3 for ln in text.splitlines()[2:])
    back = W.parse_worklist(text)
    assert back.jobs == wl.jobs and back.ranges == wl.ranges
    n = W.run_jobs(back.jobs, needD, str(tmp_path), None, ranges=back.ranges, range_fn=oracle_range(oracle))
    assert n == len(wl.jobs)
    total, counts = W.workdir_sum(str(tmp_path))
    assert sum(counts) == len(wl.jobs)
    assert total == load_golden("oracle_small.json")["100000"]["hex192"]


def test_shard_covers_disjointly():
    from clbellard_gb300 import workmode as W
    jobs = W.all_jobs(10 ** 6, 1000)
    parts = [W.shard(jobs, r, 3) for r in range(3)]
    assert sorted(j for p in parts for j in p) == sorted(jobs)
    assert sum(len(p) for p in parts) == len(jobs)


def _rank_main(rank, world, port, needD, bs, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from clbellard_gb300 import workmode as W
        from workmode_helpers import oracle_job
        d, _ = oracle.pos_to_d(needD)
        fn = oracle_job(oracle, bs)
        mine = [fn(needD, s, b, bs) for s, b in W.shard(W.all_jobs(d, bs), rank, world)]
        total = W.distributed_sum([h for h in mine if h is not None])
        out_q.put((rank, total))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_merge(oracle):
    """Two CPU ranks shard the jobs, exchange 48-hex partials (the only
    exchange step) and both obtain the single-process result."""
    import multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    needD, bs = 10000, 997
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, needD, bs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    d, _ = oracle.pos_to_d(needD)
    want = oracle.to_hex(oracle.result(d, 0, 3), 3)
    assert res[0] == res[1] == want


def test_driver_plan_worklist(cbl, oracle):
    """`cbl plan` (no GPU needed) prints a worklist the parser reads back: the
    reference's header lines, then `s_b k0 k1` lines tiling each series."""
    import subprocess
    from clbellard_gb300 import build
    from clbellard_gb300 import workmode as W
    out = subprocess.run([build.DRIVER, "plan", "1000000", "20"], capture_output=True, text=True, check=True).stdout
    wl = W.parse_worklist(out)
    d, _ = oracle.pos_to_d(1000000)
    assert wl.digits == 1000000 and wl.precision == 1 and len(wl.jobs) == 20
    assert [(s, k0, k1) for (s, _), (k0, k1) in wl.ranges.items()] == cbl.plan_jobs(1000000, 20)
    for s in range(7):
        rs = sorted(r for (f, _), r in wl.ranges.items() if f == s)
        assert rs[0][0] == 0 and rs[-1][1] == d + 20 and all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
    r = subprocess.run([build.DRIVER, "plan", "1000000", "3"], capture_output=True, text=True)
    assert r.returncode != 0
