"""Seeded random positions against the oracle, bit for bit: one batched launch
of many uneven positions (the persistent work-stealing path with all the
residue kinds below 2^32 and interleaved ladder pairs), and any-position
results with their shifted windows."""
import math
import random

import pytest

pytestmark = pytest.mark.gpu


def test_random_batched_positions(ctx192, oracle):
    rng = random.Random(0xB17E)
    pos = sorted({int(math.exp(rng.uniform(math.log(5), math.log(3e6)))) for _ in range(96)})
    got = ctx192.batch(pos)
    for p, g in zip(pos, got):
        d, _ = oracle.pos_to_d(p)
        assert g == oracle.result(d, 0, 3), p


def test_random_any_positions(ctx192, oracle):
    rng = random.Random(0xC0FFEE)
    for _ in range(24):
        p = rng.randrange(3, 2000000)
        d, sh = oracle.hexpos_to_d(p)
        assert ctx192.compute_hexpos(p) == oracle.to_hex(oracle.result(d, sh, 3), 3), p
