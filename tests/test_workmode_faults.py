"""Failure injection for work mode, on the host only: truncated and corrupt
job files, a job process killed before its file is complete, and a rank that
drops out before the merge. Nothing here touches a GPU. Recovery is the
reference's file model (a finished job is one whose file exists,
Bellard_192.hsp:307-308), tightened so a damaged file counts as not done."""
import datetime
import os

import pytest

from conftest import load_golden
from workmode_helpers import oracle_job

NEED_D, BS = 100000, 7919


def want():
    return load_golden("oracle_small.json")[str(NEED_D)]["hex192"]


def jobs(oracle):
    from clbellard_gb300 import workmode as W
    d, _ = oracle.pos_to_d(NEED_D)
    return W.all_jobs(d, BS)


@pytest.mark.parametrize("damage", [b"0123456789abcdef", b"", b"zz" * 24 + b"\r\n0\tx\r\n5ms"])
def test_damaged_job_file_is_rerun(tmp_path, cbl, oracle, damage):
    """A truncated, empty or non-hex job file reads as not done; the merge
    refuses it; run_jobs runs that job again and the merge is then exact."""
    from clbellard_gb300 import workmode as W
    js = jobs(oracle)
    fn = oracle_job(oracle, BS)
    assert W.run_jobs(js, NEED_D, str(tmp_path), fn, batchsize=BS) == len(js)
    victim = js[len(js) // 2]
    with open(W.job_path(str(tmp_path), *victim), "wb") as f:
        f.write(damage)
    assert W.read_job(str(tmp_path), *victim) is None
    with pytest.raises(cbl.CblError) as e:
        W.workdir_sum(str(tmp_path))
    assert e.value.code == -10                        # CBL_E_FORMAT
    assert W.run_jobs(js, NEED_D, str(tmp_path), fn, batchsize=BS) == 1
    total, counts = W.workdir_sum(str(tmp_path))
    assert total == want() and sum(counts) == len(js)


def test_job_write_leaves_no_partial_file(tmp_path, cbl, oracle):
    """Job files are renamed into place: no temporary remains after a write,
    and a temporary left by a killed writer is ignored by reads and the merge."""
    from clbellard_gb300 import workmode as W
    js = jobs(oracle)
    fn = oracle_job(oracle, BS)
    W.run_jobs(js, NEED_D, str(tmp_path), fn, batchsize=BS)
    for s in range(7):
        assert all(".tmp" not in n for n in os.listdir(tmp_path / str(s)))
    # a writer killed mid-write: its temporary holds half a line, the job file is absent
    s, b = js[-1]
    os.remove(W.job_path(str(tmp_path), s, b))
    with open(W.job_path(str(tmp_path), s, b) + ".tmp4242", "wb") as f:
        f.write(b"0123456789abcdef01234")
    assert W.read_job(str(tmp_path), s, b) is None
    total, counts = W.workdir_sum(str(tmp_path))       # the merge sees one job fewer
    assert counts[s] == sum(1 for j in js if j[0] == s) - 1 and total != want()
    assert W.run_jobs(js, NEED_D, str(tmp_path), fn, batchsize=BS) == 1
    assert W.workdir_sum(str(tmp_path))[0] == want()


def _rank_main(rank, world, port, workdir, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=20))
    from oracle import oracle
    from clbellard_gb300 import workmode as W
    from workmode_helpers import oracle_job
    d, _ = oracle.pos_to_d(NEED_D)
    mine = W.shard(W.all_jobs(d, BS), rank, world)
    if rank == 1:
        # dies after finishing half of its jobs, before the exchange step
        W.run_jobs(mine[: len(mine) // 2], NEED_D, workdir, oracle_job(oracle, BS), batchsize=BS)
        os._exit(3)
    W.run_jobs(mine, NEED_D, workdir, oracle_job(oracle, BS), batchsize=BS)
    try:
        W.distributed_sum([W.read_job(workdir, s, b) for s, b in mine])
        out_q.put((rank, "merged"))
    except Exception as e:                            # the peer is gone: the collective fails
        out_q.put((rank, "failed: " + type(e).__name__))
    finally:
        try:
            dist.destroy_process_group()
        except Exception:
            pass


def test_rank_drop_out_then_recover(tmp_path, cbl, oracle):
    """Rank 1 exits after half its jobs. Rank 0's merge fails with an error
    (no hang), and a rerun over the shared work directory runs exactly the
    missing jobs and gives the single-process bits."""
    import multiprocessing as mp
    import socket
    from clbellard_gb300 import workmode as W
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path), q)) for r in range(2)]
    for p in procs:
        p.start()
    rank, status = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
    assert rank == 0 and status.startswith("failed")
    assert procs[1].exitcode == 3 and procs[0].exitcode == 0
    js = jobs(oracle)
    lost = W.shard(js, 1, 2)
    missing = len(lost) - len(lost) // 2
    assert W.run_jobs(js, NEED_D, str(tmp_path), oracle_job(oracle, BS), batchsize=BS) == missing
    total, counts = W.workdir_sum(str(tmp_path))
    assert total == want() and sum(counts) == len(js)
