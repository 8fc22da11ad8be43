"""The batched-positions workload in full: 4096 reference positions drawn
log-uniform in [1e3, 1e9] (numpy default_rng(4096), as bench.py), about
8.3e11 terms, in one persistent launch. Every position <= 1e5 and 16 seeded
positions in (1e5, 1e7] are checked against the oracle; the 8 largest
(near 1e9) against single-position cbl_compute, which the 1e9/1e10 tests pin
to the oracle fixtures."""
import random

import pytest

pytestmark = pytest.mark.gpu


def positions(n=4096, seed=4096):
    import numpy as np
    rng = np.random.default_rng(seed)
    return [int(x) for x in np.rint(10.0 ** rng.uniform(3.0, 9.0, size=n))]


def test_4096_positions_one_launch(cbl, oracle):
    pos = positions()
    with cbl.Context(0, 1) as ctx:
        got = ctx.batch(pos)
        largest = sorted(range(len(pos)), key=lambda i: -pos[i])[:8]
        for i in largest:
            assert "%048x" % got[i] == ctx.compute(pos[i]), pos[i]
    small = [i for i, p in enumerate(pos) if p <= 10 ** 5]
    assert len(small) > 1000
    for i in small:
        d, _ = oracle.pos_to_d(pos[i])
        assert got[i] == oracle.result(d, 0, 3), pos[i]
    mid = [i for i, p in enumerate(pos) if 10 ** 5 < p <= 10 ** 7]
    for i in random.Random(7).sample(mid, 16):
        d, _ = oracle.pos_to_d(pos[i])
        assert got[i] == oracle.result(d, 0, 3), pos[i]
