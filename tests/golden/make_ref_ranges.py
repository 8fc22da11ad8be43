"""Generate tests/golden/ref_ranges.json: per-series partial sums over short
k-ranges computed by the reference's own kernels (Bellard.cl,
Bellard_div2by1.cl compiled as C++ by oracle/ref_harness; the -DOVERDOUBLE
build where the reference's host selects it), at positions up to the
reference's limit. Needs the reference tree; the tests read the JSON.

Each record is one BatchCalc of one series (KernelFuncs.as:25-66) followed by
Ssum and read before Sum7: the un-weighted partial bigSum[0..2] (modes 1-2, 48
hex) or the double-double pair (mode 0). "exact" marks ranges whose every
modulus is >= 2^32 and which stop below d: there mode 2 runs only the
reference's exact integer kernel (Sglobal64mtg_192_Refresh), so its partial is
an exact floor sum; elsewhere the reference's dd-based 32-bit kernel or tail
contributes and the partial is approximate.

    python tests/golden/make_ref_ranges.py
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_harness import build as R  # noqa: E402

DEN0 = (4, 4, 10, 10, 10, 10, 10)
DEN1 = (1, 3, 1, 3, 5, 7, 9)
POSITIONS = [10 ** 10, 10 ** 11, 10 ** 13, 10 ** 16, 999999999999999995]
N = 2048


def pos_to_d(needD):
    d = ((needD - 1) * 2 - 3) // 5
    return d - 1 if d % 2 == 0 else d


def first_k(f, m):
    """Smallest k with DEN0[f] k + DEN1[f] >= m."""
    return max(0, (m - DEN1[f] + DEN0[f] - 1) // DEN0[f])


def ranges(needD, f):
    d = pos_to_d(needD)
    k32, k53 = first_k(f, 1 << 32), first_k(f, 1 << 53)
    out = [("below_d", d - 3 * N, d - 2 * N, True), ("tail", d - N // 2, d, False)]
    if k32 + 4 * N < d:
        out += [("above_2^32", k32 + 2 * N, k32 + 3 * N, True), ("across_2^32", k32 - N // 2, k32 + N // 2, False)]
    if k53 + 4 * N < d:
        out += [("across_2^53", k53 - N // 2, k53 + N // 2, True)]
    return out


def main():
    recs = []
    for needD in POSITIONS:
        for f in range(7):
            for name, k0, k1, exact in ranges(needD, f):
                rec = {"needD": needD, "f": f, "range": name, "k0": k0, "k1": k1, "exact": exact}
                for prec in (0, 1, 2):
                    r = R.run_range(needD, prec, f, k0, k1)
                    rec["d"] = r["d"]
                    rec["overdouble"] = r["overdouble"]
                    p = r["partial"]
                    rec["mode%d" % prec] = list(p) if prec == 0 else "%048x" % p
                recs.append(rec)
                print(needD, f, name, rec["mode2"][:16], flush=True)
    data = {"source": ("reference kernels Bellard.cl / Bellard_div2by1.cl compiled as C++ (oracle/ref_harness), "
                       "one series' BatchCalc + Ssum per record, 64 work-groups x 256 work-items"),
            "records": recs}
    with open(os.path.join(HERE, "ref_ranges.json"), "w") as fo:
        json.dump(data, fo, indent=1)


if __name__ == "__main__":
    main()
