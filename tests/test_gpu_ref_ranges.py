"""The GPU kernels against the reference's own kernels, range by range: the
per-series partials (one BatchCalc + Ssum) recorded from Bellard.cl /
Bellard_div2by1.cl compiled as C++, at positions 1e10 ... 999999999999999995
(moduli up to 2^62)."""
from fractions import Fraction

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _ulp_dist(a, b, bits=192):
    t = (a - b) % (1 << bits)
    return min(t, (1 << bits) - t)


def records():
    return load_golden("ref_ranges.json")["records"]


def test_192bit_partials_equal_reference_exact_kernel(ctx192):
    """Where the reference runs only its exact integer kernel (every modulus
    >= 2^32, the range below d), the 192-bit partials are identical; elsewhere
    they are within 64 units of 2^-192 of the reference's dd-based pieces."""
    n_exact = 0
    for r in records():
        ctx192.Set0mem()
        ctx192.BatchCalc(r["k0"], r["k1"], r["f"], r["d"])
        got = ctx192.read_partial()
        want = int(r["mode2"], 16)
        if r["exact"]:
            assert got == want, r
            n_exact += 1
        else:
            assert _ulp_dist(got, want) <= 64, r
    assert n_exact >= 70


def test_dd_partials_against_reference_mode0(ctxdd):
    """The dd mode against the reference's mode 0 (its OVERDOUBLE build from
    2^53 on): within 2^-95 on every range."""
    for r in records():
        ctxdd.Set0mem()
        ctxdd.BatchCalc(r["k0"], r["k1"], r["f"], r["d"])
        hi, lo = ctxdd.read_partial()
        rhi, rlo = r["mode0"]
        t = ((Fraction(hi) + Fraction(lo)) - (Fraction(rhi) + Fraction(rlo))) % 1
        assert min(t, 1 - t) < Fraction(1, 2 ** 95), r
