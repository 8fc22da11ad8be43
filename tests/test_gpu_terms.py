"""Per-term parity of the CUDA term kernels with the oracle: every signed
192-bit term bit-exact, over both residue widths, their boundary, the tail,
and seeded samples of the benchmark positions."""
import random

import pytest

pytestmark = pytest.mark.gpu

W1_MAX = 1 << 28


def check_terms(ctx, oracle, d, f, ks):
    got = ctx.terms(d, f, ks)
    for k, g in zip(ks, got):
        assert g == oracle.term(d, f, k, 3), (d, f, k)


@pytest.mark.parametrize("f", range(7))
def test_terms_small_positions(ctx192, oracle, f):
    for d in (1, 3, 5, 99, 399999):
        ks = sorted(set([0, 1, 2, d - 1] + list(range(d, d + 30)) + [random.Random(d).randrange(d) for _ in range(50)]))
        check_terms(ctx192, oracle, d, f, [k for k in ks if k >= 0])


@pytest.mark.parametrize("f", range(7))
def test_terms_width_boundary(ctx192, oracle, f):
    """k around the first modulus >= 2^28 (width 1 -> middle width 1)."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    kw = (W1_MAX - den1 + den0 - 1) // den0
    d = 3999999999
    ks = list(range(kw - 40, kw + 40))
    check_terms(ctx192, oracle, d, f, ks)


@pytest.mark.parametrize("f", range(7))
def test_terms_30bit(ctx192, oracle, f):
    """k around m = 2^30 inside the middle width-1 kind, with d just either
    side so the tails fall there too."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k30 = ((1 << 30) - den1 + den0 - 1) // den0
    for d in (3999999999, k30 - 7, k30 + 3):
        check_terms(ctx192, oracle, d, f, [k for k in range(k30 - 40, k30 + 40) if k < d + 20])


@pytest.mark.parametrize("f", range(7))
def test_terms_31bit_boundary(ctx192, oracle, f):
    """k around the first modulus >= 2^31 (middle -> strict width 1)."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k31 = ((1 << 31) - den1 + den0 - 1) // den0
    for d in (3999999999, k31 + 3, k31 + 40):
        check_terms(ctx192, oracle, d, f, [k for k in range(k31 - 40, k31 + 40) if k < d + 20])


@pytest.mark.parametrize("f", range(7))
def test_terms_32bit_boundary(ctx192, oracle, f):
    """k around the first modulus >= 2^32 (strict width 1 -> width 2)."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k32 = ((1 << 32) - den1 + den0 - 1) // den0
    d = 3999999999
    check_terms(ctx192, oracle, d, f, list(range(k32 - 40, k32 + 40)))


@pytest.mark.parametrize("f", range(7))
def test_terms_40bit(ctx192, oracle, f):
    """k around m = 2^40, inside the short width-2 kind (its top words up to
    2^8 / 2^10 there), and the last terms of position 1e12."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k40 = ((1 << 40) - den1 + den0 - 1) // den0
    d = 399999999999
    check_terms(ctx192, oracle, d, f, list(range(k40 - 40, k40 + 40)) + list(range(d - 40, d + 20)))


@pytest.mark.parametrize("f", range(7))
def test_terms_44bit_boundary(ctx192, oracle, f):
    """k around the first modulus >= 2^44 (short width 2 -> width 2), where
    the short kind's top words are largest, and the last terms below d."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k44 = ((1 << 44) - den1 + den0 - 1) // den0
    d = 39999999999999
    check_terms(ctx192, oracle, d, f, list(range(k44 - 60, k44 + 40)) + list(range(d - 40, d + 20)))


def test_terms_sampled_1e8(ctx192, oracle):
    """1e5 seeded n at position 1e8 (all moduli < 2^32), all 7 series."""
    rng = random.Random(0x5EED)
    d = 39999999
    for f in range(7):
        ks = [rng.randrange(0, d + 20) for _ in range(100000 // 7)]
        check_terms(ctx192, oracle, d, f, ks)


@pytest.mark.parametrize("d", [3999999999, 39999999999, 399999999999, 399999999999999, 39999999999999999,
                               115000000000000000, 399999999999999997])
def test_terms_sampled_large(ctx192, oracle, d):
    """Positions 1e10 .. 999999999999999995 (the reference's largest): moduli
    up to ~2^61.8, exponents up to ~2^62."""
    rng = random.Random(d)
    for f in range(7):
        ks = [rng.randrange(0, d) for _ in range(3000)] + [d - 1, d - 2, d, d + 19]
        check_terms(ctx192, oracle, d, f, ks)


def test_terms_reject_modulus_range(ctx192, cbl):
    with pytest.raises(cbl.CblError) as e:
        ctx192.terms(1 << 63, 0, [1 << 60])         # 4k + 1 >= 2^62
    assert e.value.code == -6


@pytest.mark.parametrize("f", range(7))
def test_terms_60bit_boundary(ctx192, oracle, f):
    """k around the first modulus >= 2^60 (width 2 -> wide width 2)."""
    den0, den1 = oracle.DEN0[f], oracle.DEN1[f]
    k60 = ((1 << 60) - den1 + den0 - 1) // den0
    d = 399999999999999997
    check_terms(ctx192, oracle, d, f, list(range(k60 - 40, k60 + 40)) + list(range(d - 40, d + 20)))


def test_position_limits(ctx192, ctxdd, cbl):
    for ctx in (ctx192, ctxdd):
        with pytest.raises(cbl.CblError) as e:
            ctx.compute(10 ** 18)                    # above the reference's limit
        assert e.value.code == -2
