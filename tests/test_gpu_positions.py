"""Full-position parity of the CUDA path (192-bit integer mode) with the
oracle: bit-exact 192-bit results, the reference's kernel-by-kernel flow,
work-mode jobs, batched positions and overlapping positions."""
import os
import random

import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu


def agree(a, b):
    from oracle.oracle import agreeing_hex_digits
    return agreeing_hex_digits(a, b)


def test_small_positions_bit_exact(ctx192):
    g = load_golden("oracle_small.json")
    for p, v in g.items():
        assert ctx192.compute(int(p)) == v["hex192"], p


def test_precision_2_equals_1(ctx_beta):
    g = load_golden("oracle_small.json")
    for p in ("1000", "1000000"):
        assert ctx_beta.compute(int(p)) == g[p]["hex192"]


def test_1e8_against_oracle(ctx192):
    s = load_golden("recorded_probe.json")
    pub = load_golden("published_digits.json")["digits"]
    h = ctx192.compute(10 ** 8)
    assert h.startswith(pub["100000000"])
    assert agree(h, s["exact256"]["100000000"]) >= 36
    # the reference's own 192-bit output (CPU-run kernels) agrees for >= 24 digits
    assert agree(h, s["ref_mode2"]["100000000"]) >= 24
    path = os.path.join(GOLDEN, "oracle_big.json")
    if os.path.exists(path):
        big = load_golden("oracle_big.json")
        if "100000000" in big:
            assert h == big["100000000"]["hex192"]


def test_reference_kernel_flow_equals_compute(ctx192, oracle):
    """Set0mem / BatchCalc / AddAns per series (Bellard_192.hsp:264-296)."""
    needD = 123455
    d, _ = oracle.pos_to_d(needD)
    ctx192.Set0ans()
    for f in range(7):
        ctx192.Set0mem()
        ctx192.BatchCalc(0, d, f, d)
        ctx192.AddAns(f)
        # the weighted partial written back equals the oracle's series << numer
        assert ctx192.read_partial() == (oracle.series(d, f, 3) << oracle.NUMER_LOG2[f]) % (1 << 192)
    ans = ctx192.read_ans()
    assert "%048x" % ans == oracle.to_hex(oracle.result(d, 0, 3), 3) == ctx192.compute(needD)


def test_sglobal_split_32_64(ctx192, oracle):
    """KernelFuncs.as:25-66 by hand: the 32-bit range, the 64-bit range, the
    tail, Ssum; split at the m = 2^32 boundary of series 2 at 1e10."""
    d = 3999999999
    f = 2
    _, sign, den0, den1 = 256, 0, 10, 1
    k32 = ((1 << 32) - den1 - 1) // den0 + 1
    ka, kb = k32 - 3000, k32 + 5000
    ctx192.Set0mem()
    ctx192.Sglobal32mtg(ka, d, k32, sign, den0, den1)
    ctx192.Sglobal64mtg(k32, d, kb, sign, den0, den1)
    ctx192.Ssum()
    assert ctx192.read_partial() == oracle.sum_range(d, f, ka, kb, 3)
    ctx192.Set0mem()
    ctx192.Sglobal_after(d, sign, den0, den1)
    ctx192.Ssum()
    assert ctx192.read_partial() == oracle.sum_range(d, f, d, d + 20, 3)


def test_sglobal_range_errors(ctx192, cbl):
    d = 3999999999
    with pytest.raises(cbl.CblError) as e:
        ctx192.Sglobal32mtg(429496729, d, 429496731, 0, 10, 1)      # m >= 2^32
    assert e.value.code == -6
    with pytest.raises(cbl.CblError) as e:
        ctx192.Sglobal64mtg(0, 100, 101, 0, 10, 1)                 # k_max > d
    assert e.value.code == -6
    with pytest.raises(cbl.CblError):
        ctx192.Sglobal64mtg(0, 100, 50, 0, 10, 2)                  # even moduli
    with pytest.raises(cbl.CblError):
        ctx192.Sum7(3)


def test_workmode_jobs_sum_to_result(ctx192, tmp_path, oracle):
    from clbellard_gb300 import workmode as W
    needD = 1000000
    d, _ = oracle.pos_to_d(needD)
    bs = 65521
    jobs = W.all_jobs(d, bs)
    W.run_jobs(jobs, needD, str(tmp_path), W.gpu_job_fn(ctx192), batchsize=bs, devname=ctx192.device_name)
    total, counts = W.workdir_sum(str(tmp_path))
    assert total == ctx192.compute(needD) == load_golden("oracle_small.json")["1000000"]["hex192"]
    assert ctx192.run_job(needD, 0, d // bs + 1, bs) is None          # k_start > d: skipped


def test_balanced_jobs_sum_to_result(ctx192, tmp_path):
    """Balanced explicit-range jobs (cbl_plan_jobs) merged equal normal mode."""
    from clbellard_gb300 import workmode as W
    needD = 10 ** 7
    wl = W.balanced_worklist(needD, 20)
    W.run_jobs(wl.jobs, needD, str(tmp_path), W.gpu_job_fn(ctx192), ranges=wl.ranges,
               range_fn=W.gpu_range_fn(ctx192), devname=ctx192.device_name)
    total, counts = W.workdir_sum(str(tmp_path))
    assert sum(counts) == 20
    assert total == ctx192.compute(needD) == load_golden("oracle_small.json")[str(needD)]["hex192"]


def test_job_range_matches_oracle(ctx192, oracle):
    needD = 100000
    d, _ = oracle.pos_to_d(needD)
    for s, k0, k1 in [(0, 0, 1), (3, 17, 9001), (6, 39000, d), (2, d - 5, d + 20), (5, 0, d + 20)]:
        kend = min(k1, d)
        v = oracle.sum_range(d, s, k0, kend, 3) if k0 < kend else 0
        if max(k0, kend) == d:
            v += oracle.sum_range(d, s, d, d + 20, 3)
        assert ctx192.run_job_range(needD, s, k0, k1) == "%048x" % ((v << oracle.NUMER_LOG2[s]) % (1 << 192))
    assert ctx192.run_job_range(needD, 0, d + 1, d + 20) is None


def test_default_batch_jobs(ctx192, oracle):
    """The reference's 2^37 batch: one job per series covers d < 2^37."""
    needD = 10000
    d, _ = oracle.pos_to_d(needD)
    hs = [ctx192.run_job(needD, s, 0) for s in range(7)]
    from clbellard_gb300 import workmode_sum
    assert workmode_sum(hs) == oracle.to_hex(oracle.result(d, 0, 3), 3)


def test_batched_positions(ctx192, oracle):
    """Many uneven positions in one persistent launch (log-uniform, seeded)."""
    import math
    rng = random.Random(4096)
    pos = sorted(int(10 ** rng.uniform(3, 5.3)) for _ in range(48)) + [5, 10, 15]
    got = ctx192.batch(pos)
    for p, g in zip(pos, got):
        d, _ = oracle.pos_to_d(p)
        assert g == oracle.result(d, 0, 3), p


def test_hexpos_any_position(ctx192, oracle):
    for p in (3, 4, 6, 7, 11, 1001, 99999, 123457):
        d, sh = oracle.hexpos_to_d(p)
        assert ctx192.compute_hexpos(p) == oracle.to_hex(oracle.result(d, sh, 3), 3), p


def test_overlap_p_and_p_minus_8(ctx192):
    """Digits of position P-8 shifted by 8 agree with position P."""
    for P in (10 ** 6, 10 ** 8):
        a = ctx192.compute_hexpos(P)
        b = ctx192.compute_hexpos(P - 8)
        assert agree(a, b[8:]) >= 28


def test_tuning_does_not_change_bits(ctx192):
    ref = ctx192.compute(10 ** 6)
    for tile, ctas in ((32, 1), (96, 3), (4096, 0), (2048, 0)):
        ctx192.set_tuning(tile, ctas)
        assert ctx192.compute(10 ** 6) == ref
    ctx192.set_tuning(2048, 0)


def test_query_wait(ctx192):
    ctx192.prepare([10 ** 7])
    ctx192.run_prepared()
    ctx192.wait(60000)
    assert ctx192.query() == 0
    d = 3999999
    assert ctx192.read_results()[0] == int(load_golden("oracle_small.json")["10000000"]["hex192"], 16)


def test_launch_count_counts_kernels(ctx192):
    ctx192.prepare([10 ** 5])
    n0 = ctx192.launch_count
    ctx192.run_prepared()
    ctx192.wait()
    assert ctx192.launch_count - n0 == 2


def test_against_reference_kernels(ctx192, ctxdd):
    """GPU results against the reference's own kernels run on the CPU (up to
    position 1e10 in full): the 192-bit modes agree for >= 24 hex digits (the
    target for this path), the 106-bit mode for >= 19."""
    ref = load_golden("ref_outputs.json")
    for p, e in ref.items():
        if not p.isdigit():
            continue
        h = ctx192.compute(int(p))
        for mode in ("mode1", "mode2"):
            if mode in e:
                assert agree(h, e[mode]) >= 24, (p, mode)
        if "mode0" in e:
            assert agree(ctxdd.compute(int(p)), e["mode0"]) >= 19, p


def test_autotune_keeps_bits(cbl, tmp_path, monkeypatch):
    monkeypatch.setenv("CBL_TUNE_CACHE", str(tmp_path / "tune.txt"))
    pos = [1000, 123455, 10 ** 6]
    with cbl.Context(0, 1) as ctx:
        want = ctx.batch(pos)
        tile, ctas, ms = ctx.autotune(pos, force=True)
        assert tile in (512, 1024, 2048, 4096, 8192) and ctas >= 1 and ms > 0
        ctx.run_prepared()
        ctx.wait()
        assert ctx.read_results() == want
        assert (tmp_path / "tune.txt").exists()
        t2, c2, ms2 = ctx.autotune(pos)              # served from the cache
        assert (t2, c2, ms2) == (tile, ctas, -1.0)
