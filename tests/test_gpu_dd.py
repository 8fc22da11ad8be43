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


def _dd_mod1(hi, lo):
    from fractions import Fraction
    return (Fraction(hi) + Fraction(lo)) % 1


def _close_mod1(x, y, tol):
    t = (x - y) % 1
    return min(t, 1 - t) < tol


@pytest.mark.parametrize("needD", [10 ** 16, 999999999999999995])
def test_dd_overdouble_against_exact(ctxdd, oracle, needD):
    """Moduli >= 2^53 in mode 0 (the reference's OVERDOUBLE build): r and m
    as exact double-doubles, divided in double-double. Sampled ranges just
    across 2^53, just below d (up to 2^62 near the position limit) and the
    10-term tail agree with the exact 256-bit oracle to 2^-90."""
    from fractions import Fraction
    d, _ = oracle.pos_to_d(needD)
    tol = Fraction(1, 2 ** 90)
    for f in range(7):
        den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
        k53 = ((1 << 53) - den1 + den0 - 1) // den0
        for k0, k1 in [(k53 - 2048, k53 + 2048), (d - 4096, d - 1)]:     # k1 < d: no tail here
            ctxdd.Set0mem()
            ctxdd.BatchCalc(k0, k1, f, d)
            got = _dd_mod1(*ctxdd.read_partial())
            want = Fraction(oracle.sum_range(d, f, k0, k1, 4), 2 ** 256)
            assert _close_mod1(got, want, tol), (f, k0, float((got - want) % 1))
        ctxdd.Set0mem()
        ctxdd.Sglobal_after(d, oracle.SIGN[f], den0, den1)
        ctxdd.Ssum()
        got = _dd_mod1(*ctxdd.read_partial())
        want = Fraction(oracle.sum_range(d, f, d, d + 10, 4), 2 ** 256)
        assert _close_mod1(got, want, tol), (f, "tail")
