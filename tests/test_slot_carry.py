"""The carry rule of the term kernel's digit-sum slots, restated on the CPU.

A slot holds six 64-bit sums, element j weighing 2^(32j). Flushing a tile adds
a normalised 32-bit digit to each element; when such an add wraps element j
past 2^64 the kernel adds one unit to element j+2 (2^64 * 2^(32j) =
2^(32(j+2))), repeating on a further wrap, and drops carries from element 6
on (weight >= 2^192). This test checks that the rule keeps the slot's value
equal to the exact sum mod 2^192 for any number of adds and any start value,
so no position needs a bound on tiles per slot."""
import random

M64 = (1 << 64) - 1
M192 = (1 << 192) - 1


def slot_add(slot, j, v):
    while True:
        old = slot[j]
        slot[j] = (old + v) & M64
        if old + v <= M64:
            return
        j += 2
        v = 1
        if j >= 6:
            return


def value(slot):
    return sum(s << (32 * j) for j, s in enumerate(slot)) & M192


def test_carry_rule_exact_over_many_wraps():
    rng = random.Random(7)
    for start in ([M64] * 6, [M64 - (1 << 33)] * 6, [rng.getrandbits(64) for _ in range(6)], [0] * 6):
        slot = list(start)
        want = value(slot)
        for _ in range(20000):
            tile = rng.getrandbits(192)                       # one tile's 192-bit warp sum
            for j in range(6):
                dj = (tile >> (32 * j)) & 0xffffffff
                if dj:
                    slot_add(slot, j, dj)
            want = (want + tile) & M192
        assert value(slot) == want


def test_no_carry_loses_value_beyond_2_32_tiles():
    """Without the carry a slot whose elements reach 2^64 loses 2^64 per wrap:
    the rule is needed once a slot takes 2^32 tiles of near-full digits."""
    slot = [M64 - 5] * 6
    plain = [(s + 10) & M64 for s in slot]
    assert value(plain) != (value(slot) + sum(10 << (32 * j) for j in range(6))) & M192
    for j in range(6):
        slot_add(slot, j, 10)
    assert value(slot) == (value([M64 - 5] * 6) + sum(10 << (32 * j) for j in range(6))) & M192
