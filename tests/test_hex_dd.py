"""The mode-0 printer: cbl_hex_dd against the reference's hexadecimal_dd
(hexsademical.as:21-101, restated in oracle.hexadecimal_dd).

The reference lifts a negative value by 1.0 with its double-double add, then
scales by 256 fourteen times and takes the integer part as the next byte. The
scaling and renormalisation are exact, so its bytes are the exact 112-bit
truncation of the lifted value except after a negative intermediate byte.
There its borrow branch (hexsademical.as:73-97) keeps x + 256 as the remainder
instead of reducing it, and every later byte prints as 00. cbl_hex_dd performs
the same lift and then the exact truncation: byte for byte the reference's
output wherever that branch is not taken, the value's own bytes where it is
(a deliberate fix)."""
import random

import pytest

from conftest import load_golden


def _pairs_random(seed, n, negative_lo=False):
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        hi = rng.random() * rng.choice((1.0, -1.0))
        lo = (rng.random() - 0.5) * 2.0 ** -53 * abs(hi)
        out.append((hi, -abs(lo) if negative_lo else lo))
    return out


def _near_boundaries():
    cases = []
    for b in range(1, 14):                          # just below and on byte boundaries
        for top in (0x01, 0x3b, 0x7f, 0xff):
            hi = (top + 1) / 256.0 - 2.0 ** (-8 * b)
            if hi >= 1.0:                           # 1 - 2^-104 rounds to 1.0
                continue
            cases += [(hi, 2.0 ** (-8 * b - 60)), (hi, 2.0 ** (-8 * b - 60) * 0.75),
                      (-hi, -2.0 ** (-8 * b - 60)), (hi, -2.0 ** (-8 * b - 60))]
    return cases


def test_restated_printer_is_the_lifted_exact_truncation(oracle):
    """Where the borrow branch is not taken, the restated printer's bytes are
    the exact truncation of the (lifted) value."""
    n = 0
    for hi, lo in _pairs_random(21, 4000) + _pairs_random(22, 2000, negative_lo=True) + _near_boundaries():
        h, borrowed = oracle.hexadecimal_dd(hi, lo, report=True)
        if not borrowed:
            assert h == oracle.dd_exact_hex(hi, lo, lift=True), (hi, lo)
            n += 1
    assert n > 5500


def test_hex_dd_equals_reference_printer_on_reference_mode0_values(cbl, oracle):
    """The reference's own mode-0 values: the per-series partials of the
    reference kernels (ref_ranges.json) and full results (ref_outputs.json),
    whose mode0 strings are the reference printer's output."""
    pairs = [tuple(r["mode0"]) for r in load_golden("ref_ranges.json")["records"] if "mode0" in r]
    outs = load_golden("ref_outputs.json")
    full = {k: (float.fromhex(v["mode0_dd"][0]), float.fromhex(v["mode0_dd"][1]))
            for k, v in outs.items() if isinstance(v, dict) and "mode0_dd" in v}
    assert len(full) >= 5
    pairs += list(full.values())
    assert len(pairs) >= 100
    for hi, lo in pairs:
        h, borrowed = oracle.hexadecimal_dd(hi, lo, report=True)
        assert not borrowed
        assert cbl.hex_dd(hi, lo) == h, (hi, lo)
    for k, (hi, lo) in full.items():
        assert cbl.hex_dd(hi, lo) == outs[k]["mode0"], k


def test_hex_dd_equals_reference_printer_random_negative_lo_and_boundaries(cbl, oracle):
    n = 0
    for hi, lo in _pairs_random(5, 3000) + _pairs_random(6, 3000, negative_lo=True) + _near_boundaries():
        h, borrowed = oracle.hexadecimal_dd(hi, lo, report=True)
        if borrowed:
            continue
        assert cbl.hex_dd(hi, lo) == h, (hi, lo)
        n += 1
    assert n > 5900


@pytest.mark.parametrize("hi,lo", [(0.5, -2.0 ** -100), (0.25, -2.0 ** -90), (0x3c / 256.0, -2.0 ** -70),
                                   (-0.5, -2.0 ** -100), (0.75, -2.0 ** -60)])
def test_borrow_branch_divergence(cbl, oracle, hi, lo):
    """hi on a byte boundary with a negative lo: the reference's borrow
    branch leaves every byte after it 00; cbl_hex_dd gives the exact value.
    Both agree up to the byte the borrow lowers."""
    ref, borrowed = oracle.hexadecimal_dd(hi, lo, report=True)
    ours, exact = cbl.hex_dd(hi, lo), oracle.dd_exact_hex(hi, lo, lift=True)
    assert borrowed and ours == exact and ref != exact
    n = oracle.agreeing_hex_digits(ref, exact)
    assert n >= 2 and set(ref[n:]) == {"0"}


def test_hex_dd_rejects_values_outside_the_unit_interval(cbl):
    for hi, lo in ((1.0, 0.0), (float("nan"), 0.0), (0.5, float("inf"))):
        with pytest.raises(cbl.CblError):
            cbl.hex_dd(hi, lo)
