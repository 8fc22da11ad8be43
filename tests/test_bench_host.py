"""bench.py's host side on the CPU: the reference arm under torchrun with two
gloo ranks (rank 0 alone runs and prints one JSON line, the other exits 0
without work), and the max-over-ranks timing of the multi-rank path."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_reference_arm_two_ranks():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--ref-seconds", "0.3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["cpu_baseline"]["kind"] in ("reference", "port") and rec["cpu_baseline"]["value"] == rec["value"]
    assert rec["e2e"]["h2d_bytes_per_step"] == 0 and rec["e2e"]["value"] == rec["value"]
    # the same config as the GPU arm, key for key; what was timed, and what is extrapolated
    sys.path.insert(0, ROOT)
    import bench
    assert rec["config"] == bench.workload_config(3999999999)
    assert rec["extrapolated"] is True and rec["timed_s"] > 0 and rec["terms_timed"] > 0
    assert abs(rec["value"] - rec["terms_timed"] / rec["timed_s"]) <= 1e-6 * rec["value"]
    assert rec["ms_per_position_extrapolated"] > rec["ms_per_step"]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    world, r, _ = bench.dist_init()
    try:
        bench.barrier(world)
        q.put((r, bench.max_over_ranks(10.0 + r, world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 11.0, 1: 11.0}


def _split_rank(rank, world, port, needD, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as O
    w, r, _ = bench.dist_init()
    d, _ = O.pos_to_d(needD)

    def run_range(s, k0, k1):
        # the oracle's partial of job (s, [k0, k1)): what cbl_run_job_range returns
        return "%048x" % ((O.sum_range(d, s, k0, k1, 3) << O.NUMER_LOG2[s]) % (1 << 192))

    try:
        q.put((r, bench.split_position(needD, w, r, run_range)))
    finally:
        if w > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


def test_split_position_two_gloo_ranks_gives_single_rank_bits(oracle):
    """bench.py's multi-GPU path: one position cut into 8 balanced jobs per
    rank, each rank runs its share, and the exact 48-hex merge over the ranks
    equals the position's result (here with the oracle standing in for the
    GPU job)."""
    import multiprocessing as mp
    needD = 123455
    d, _ = oracle.pos_to_d(needD)
    want = oracle.to_hex(oracle.result(d, 0, 3), 3)
    ctx = mp.get_context("spawn")
    for world in (1, 2):
        q = ctx.Queue()
        port = _free_port()
        procs = [ctx.Process(target=_split_rank, args=(r, world, port, needD, q)) for r in range(world)]
        for p in procs:
            p.start()
        got = dict(q.get(timeout=180) for _ in procs)
        for p in procs:
            p.join(timeout=60)
            assert p.exitcode == 0
        assert set(got.values()) == {want}, (world, got)
