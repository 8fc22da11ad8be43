"""The exact CPU oracle against the golden vectors, published digits and an
independent pure-Python restatement (all CPU)."""
import random

import pytest

from conftest import load_golden


def test_formula_table(oracle):
    # KernelFuncs.as:9-12
    assert oracle.NUMER_LOG2 == (5, 0, 8, 6, 2, 2, 0)
    assert oracle.SIGN == (1, 1, 0, 1, 1, 1, 0)
    assert oracle.DEN0 == (4, 4, 10, 10, 10, 10, 10)
    assert oracle.DEN1 == (1, 3, 1, 3, 5, 7, 9)


@pytest.mark.parametrize("needD,d,adj", [
    (5, 1, 5), (6, 1, 5), (9, 1, 5), (10, 3, 10), (12, 3, 10), (1000000, 399999, 1000000),
    (1000001, 399999, 1000000), (10000000000, 3999999999, 10000000000),
    (999999999999999999, 399999999999999997, 999999999999999995)])
def test_pos_to_d(oracle, needD, d, adj):
    # Bellard_192.hsp:468-470: d odd, needD re-derived, always a multiple of 5
    assert oracle.pos_to_d(needD) == (d, adj)
    assert d % 2 == 1 and adj % 5 == 0


@pytest.mark.parametrize("needD", [0, 1, 4, 10 ** 18])
def test_pos_to_d_invalid(oracle, needD):
    # Bellard_192.hsp:449-450
    assert oracle.pos_to_d(needD) is None


def test_hexpos_matches_reference_mapping(oracle):
    for needD in (5, 10, 1000, 10 ** 6):
        d, adj = oracle.pos_to_d(needD)
        assert oracle.hexpos_to_d(adj) == (d, 0)


def test_pow2mod_against_python(oracle):
    rng = random.Random(0x5EED)
    for _ in range(3000):
        m = rng.randrange(3, 1 << 62) | 1
        e = rng.randrange(0, 1 << 40)
        assert oracle.pow2mod(e, m) == pow(2, e, m) == oracle.pow2mod_plain(e, m)
    assert oracle.pow2mod(5, 1) == 0


def test_terms_against_python(oracle):
    rng = random.Random(7)
    for _ in range(2000):
        f = rng.randrange(7)
        d = rng.choice([1, 3, 399999, rng.randrange(1, 10 ** 11)])
        k = rng.choice([0, d - 1, d, d + 19, d + 25, rng.randrange(0, d + 30)])
        for W in (3, 4):
            assert oracle.term(d, f, k, W) == oracle.py_term(d, f, k, W), (d, f, k, W)


@pytest.mark.parametrize("d", [1, 3, 5, 39, 121])
def test_result_against_python(oracle, d):
    for W in (3, 4):
        assert oracle.result(d, 0, W) == oracle.py_result(d, 0, W)


def test_small_fixture(oracle):
    g = load_golden("oracle_small.json")
    for k, v in g.items():
        d, adj = oracle.pos_to_d(int(k))
        assert (v["d"], v["needD"]) == (d, adj)
        if d < 10 ** 6:
            assert oracle.to_hex(oracle.result(d, 0, 3), 3) == v["hex192"]
            assert oracle.to_hex(oracle.result(d, 0, 4), 4) == v["hex256"]


def test_known_pi_prefix(oracle):
    # pi = 3.243F6A8885A308D313198A2E0370734...: position 5 starts at "6A88"
    d, _ = oracle.pos_to_d(5)
    assert oracle.to_hex(oracle.result(d, 0, 4), 4).startswith("6a8885a308d313198a2e0370734")


def test_exact_oracle_against_recorded_and_published():
    g = load_golden("oracle_small.json")
    s = load_golden("recorded_probe.json")
    pub = load_golden("published_digits.json")["digits"]
    from oracle.oracle import agreeing_hex_digits as agree
    for p in ("1000000", "10000000"):
        assert agree(g[p]["hex256"], s["exact256"][p]) >= 50
        assert g[p]["hex256"].startswith(pub[p])
        # the 192-bit definition keeps >= 36 hex digits (error <= 362 d ulps)
        assert agree(g[p]["hex192"], g[p]["hex256"]) >= 36
        # the reference's 192-bit output agrees with the exact value to >= 24 digits
        assert agree(s["ref_mode2"][p], s["exact256"][p]) >= 24


def test_big_fixture_consistency():
    import os
    from conftest import GOLDEN
    from oracle.oracle import agreeing_hex_digits as agree
    path = os.path.join(GOLDEN, "oracle_big.json")
    if not os.path.exists(path):
        pytest.skip("oracle_big.json not generated")
    g = load_golden("oracle_big.json")
    s = load_golden("recorded_probe.json")
    pub = load_golden("published_digits.json")["digits"]
    for p, v in g.items():
        if p in pub:
            assert v["hex256"].startswith(pub[p])
        assert agree(v["hex192"], v["hex256"]) >= 33
        if p in s["exact256"]:
            assert agree(v["hex256"], s["exact256"][p]) >= 48


def test_hex48_sum_wraps(oracle):
    assert oracle.hex48_sum(["f" * 48, "0" * 47 + "1"]) == "0" * 48
    assert oracle.hex48_sum(["0" * 47 + "f", "0" * 47 + "1"]) == "0" * 46 + "10"
    assert oracle.hex48_sum(["0" * 47 + "g"]) is None


def test_sum_is_mod_2_192(oracle):
    # the sum of all jobs of a split equals the unsplit series (associative integer add)
    d, _ = oracle.pos_to_d(100000)
    whole = oracle.series(d, 3)
    parts = oracle.sum_range(d, 3, 0, 1000) + oracle.sum_range(d, 3, 1000, d + 20)
    assert parts % (1 << 192) == whole


def test_dd_oracle_digits_kept(oracle):
    from oracle.oracle import agreeing_hex_digits as agree
    d, _ = oracle.pos_to_d(100000)
    hi, lo = oracle.dd_result(d)
    x = (int(hi * (1 << 100)) << 92) + int(lo * (1 << 192))   # approximate 192-bit image
    exact = oracle.to_hex(oracle.result(d, 0, 4), 4)
    assert agree(format(x % (1 << 192), "048x"), exact) >= 20


def test_oracle_against_reference_kernels(oracle):
    """The reference's own kernels run on the CPU (tests/golden/ref_outputs.json,
    made by tests/golden/make_ref_golden.py) against the exact oracle."""
    from oracle.oracle import agreeing_hex_digits as agree
    ref = load_golden("ref_outputs.json")
    small = load_golden("oracle_small.json")
    big = load_golden("oracle_big.json")
    for p, e in ref.items():
        if not p.isdigit():
            continue
        d, _ = oracle.pos_to_d(int(p))
        assert e["d"] == d
        if p in small:
            exact = small[p]["hex256"]
        elif p in big:
            exact = big[p]["hex256"]
        else:
            exact = oracle.to_hex(oracle.result(d, 0, 4), 4)
        # 192-bit modes (dd pairs below 2^32, exact quotients above) keep >= 36 hex digits
        for mode in ("mode1", "mode2"):
            if mode in e:
                assert agree(e[mode], exact) >= 36, (p, mode)
        # the 106-bit mode keeps >= 20
        if "mode0" in e:
            assert agree(e["mode0"], exact) >= 20, p
            assert e["mode0"].endswith("0" * 20)


def test_reference_192bit_output_at_1e10_in_full():
    """The reference's own 192-bit kernels (precision 2, "192bit(beta)") run
    in full at position 1e10 on the CPU (Bellard_192.hsp:264-296 through
    KernelFuncs.as:25-74, Bellard_div2by1.cl:313-359 for m >= 2^32): its 48
    hex digits against the exact oracle. This is the value the GPU result is
    held to (>= 24 digits) in the GPU tests."""
    from oracle.oracle import agreeing_hex_digits as agree
    e = load_golden("ref_outputs.json")["10000000000"]
    big = load_golden("oracle_big.json")["10000000000"]
    assert e["d"] == big["d"] == 3999999999
    assert agree(e["mode2"], big["hex256"]) >= 36
    assert agree(e["mode2"], big["hex192"]) >= 36


def test_reference_outputs_match_recorded_probe():
    """The harness reproduces the recorded reference outputs (an independent earlier run)."""
    ref = load_golden("ref_outputs.json")
    s = load_golden("recorded_probe.json")
    for p, h in s["ref_mode2"].items():
        if p in ref:
            assert ref[p]["mode2"] == h
    for p, h in s["ref_mode0_prefix"].items():
        if p in ref:
            assert ref[p]["mode0"].startswith(h)


def _ref_range_exact(oracle, r):
    """The oracle's 192-bit partial for one reference range record."""
    d, f, k0, k1 = r["d"], r["f"], r["k0"], r["k1"]
    kend = min(k1, d)
    v = oracle.sum_range(d, f, k0, kend, 3) if k0 < kend else 0
    if max(k0, kend) == d:
        v += oracle.sum_range(d, f, d, d + 20, 3)
    return v % (1 << 192)


def _ulp_dist(a, b, bits=192):
    t = (a - b) % (1 << bits)
    return min(t, (1 << bits) - t)


def test_oracle_against_reference_64bit_kernels():
    """Per-series partials of the reference's own kernels over short k-ranges
    at positions 1e10 ... 999999999999999995 (moduli up to 2^62, the
    OVERDOUBLE build above 2^53): on ranges with every modulus >= 2^32 the
    reference's exact integer kernel (Sglobal64mtg_192_Refresh, mode 2)
    equals the oracle bit for bit; where its dd-based 32-bit kernel or tail
    takes part, and in mode 1, it is within 64 units of 2^-192; mode 0 (dd)
    is within 2^-96."""
    from fractions import Fraction
    from oracle import oracle
    oracle.build()
    recs = load_golden("ref_ranges.json")["records"]
    assert len(recs) >= 150 and any(r["overdouble"] for r in recs)
    n_exact = 0
    for r in recs:
        v = _ref_range_exact(oracle, r)
        m2, m1 = int(r["mode2"], 16), int(r["mode1"], 16)
        if r["exact"]:
            assert m2 == v, r
            n_exact += 1
        else:
            assert _ulp_dist(m2, v) <= 64, r
        assert _ulp_dist(m1, v) <= 64, r
        hi, lo = r["mode0"]
        t = ((Fraction(hi) + Fraction(lo)) - Fraction(v, 1 << 192)) % 1
        assert min(t, 1 - t) < Fraction(1, 2 ** 96), r
    assert n_exact >= 70
