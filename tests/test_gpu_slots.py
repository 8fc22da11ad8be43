"""Digit-sum slots that wrap past 2^64 stay exact.

Each warp flush adds six normalised 32-bit digits into a slot's six 64-bit
digit sums, so without a carry a slot would overflow after 2^32 flushes
(positions beyond about 2e13 with 2048-term tiles). When a slot may take 2^31
or more flushes, or starts from a preset, the term kernel carries a wrapped
element into element j+2. These tests start every slot from a preset near 2^64
(cbl_set_slot_preset), so the sums wrap within a few flushes, and check the
result against the oracle plus the preset's known contribution."""
import random

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

M192 = (1 << 192) - 1
NUMER_LOG2 = (5, 0, 8, 6, 2, 2, 0)


def expected(true_hex: str, preset) -> str:
    """Every series partial starts at sum_j preset[j] 2^(32j) mod 2^192, which
    the combine step weights by numer like the partial itself."""
    v = sum(int(p) << (32 * j) for j, p in enumerate(preset)) & M192
    return "%048x" % ((int(true_hex, 16) + sum(v << s for s in NUMER_LOG2)) & M192)


rng = random.Random(0x510)
PRESETS = [
    [(1 << 64) - (1 << 36)] * 6,                              # wraps after a few dozen tiles
    [(1 << 64) - 1] * 6,                                      # every add wraps, carries cascade
    [(1 << 64) - rng.getrandbits(34) for _ in range(6)],
]


@pytest.mark.parametrize("preset", PRESETS, ids=["near", "full", "random"])
def test_wrapped_slots_bit_exact(cbl, preset):
    small = load_golden("oracle_small.json")
    big = load_golden("oracle_big.json")
    with cbl.Context(0, 1) as ctx:
        ctx.set_tuning(64)                                    # small tiles: many flushes per slot
        ctx.set_slot_preset(preset)
        for p in ("1000", "1000000", "10000000"):
            assert ctx.compute(int(p)) == expected(small[p]["hex192"], preset), p
        assert ctx.compute(10 ** 8) == expected(big["100000000"]["hex192"], preset)
        pos = [1000, 10 ** 6, 10 ** 7]
        got = ctx.batch(pos)
        assert ["%048x" % x for x in got] == [expected(small[str(p)]["hex192"], preset) for p in pos]
        ctx.set_slot_preset(None)
        assert ctx.compute(10 ** 7) == small["10000000"]["hex192"]


def test_wrapped_slots_in_budgeted_passes(cbl):
    """Resumable passes clear (or preset) the slots the same way."""
    preset = PRESETS[0]
    big = load_golden("oracle_big.json")
    with cbl.Context(0, 1) as ctx:
        ctx.set_tuning(256)
        ctx.set_slot_preset(preset)
        ctx.prepare([10 ** 8])
        done = total = None
        while done is None or done < total:
            done, total = ctx.run_prepared_budget(5.0)
        assert "%048x" % ctx.read_results()[0] == expected(big["100000000"]["hex192"], preset)
