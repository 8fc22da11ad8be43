"""The 106-bit double-double mode on the GPU: digits kept against the exact
oracle, the reference's output format, and the kernel-by-kernel flow."""
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def agree(a, b):
    from oracle.oracle import agreeing_hex_digits
    return agreeing_hex_digits(a, b)


@pytest.mark.parametrize("p", ["1000", "100000", "1000000", "10000000"])
def test_dd_digits_kept(ctxdd, p):
    g = load_golden("oracle_small.json")
    h = ctxdd.compute(int(p))
    assert len(h) == 48 and h.endswith("0" * 20)        # 14 bytes + zero padding
    assert agree(h, g[p]["hex256"]) >= 20


def test_dd_1e8_vs_reference_mode0(ctxdd):
    s = load_golden("recorded_probe.json")
    h = ctxdd.compute(10 ** 8)
    assert agree(h, s["exact256"]["100000000"]) >= 19
    assert agree(h, s["ref_mode0_prefix"]["100000000"]) >= 19


def test_dd_flow_and_jobs(ctxdd, oracle):
    needD = 10000
    d, _ = oracle.pos_to_d(needD)
    ctxdd.Set0ans()
    for f in range(7):
        ctxdd.Set0mem()
        ctxdd.BatchCalc(0, d, f, d)
        ctxdd.AddAns(f)
    hi, lo = ctxdd.read_ans()
    assert 0.0 <= hi < 1.0
    exact = oracle.result(d, 0, 4)
    assert abs((hi + lo) - exact / 2.0 ** 256) < 1e-25
    h = ctxdd.run_job(needD, 3, 0)
    assert len(h) == 48
    with pytest.raises(Exception):
        ctxdd.batch([1000])
