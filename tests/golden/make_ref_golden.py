"""Generate tests/golden/ref_outputs.json by running the reference's own
kernels (compiled as C++ on the CPU by oracle/ref_harness) at several
positions in all three precision modes. Needs the reference tree; the
committed JSON is what the tests read.

    python tests/golden/make_ref_golden.py [--big]
    python tests/golden/make_ref_golden.py --positions 10000000000 --modes 2 1 0
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref_harness import build as R  # noqa: E402

POSITIONS = [1000, 10000, 100000, 1000000, 10000000]
BIG = [100000000]


def dd_hex(hi: float, lo: float) -> str:
    """The reference's mode-0 print form of its double-double result: its
    printer hexadecimal_dd (hexsademical.as:21-101) as restated in the oracle
    (28 hex digits and 20 zeros)."""
    from oracle import oracle as O
    return O.hexadecimal_dd(hi, lo)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true", help="position 1e8 (minutes)")
    ap.add_argument("--positions", type=int, nargs="*", default=None,
                    help="explicit positions (1e10: about 30 min per mode on 8 threads)")
    ap.add_argument("--modes", type=int, nargs="*", default=[0, 1, 2])
    args = ap.parse_args()
    path = os.path.join(HERE, "ref_outputs.json")
    data = json.load(open(path)) if os.path.exists(path) else {}
    data["source"] = ("reference kernels Bellard.cl / Bellard_div2by1.cl compiled as C++ (oracle/ref_harness), "
                      "64 work-groups x 256 work-items, launch sequence of KernelFuncs.as")
    positions = args.positions if args.positions else (BIG if args.big else POSITIONS)
    for p in positions:
        for prec in args.modes:
            r = R.run(p, prec, timeout=6 * 3600.0)
            data = json.load(open(path)) if os.path.exists(path) else data
            e = data.setdefault(str(p), {})
            e["d"] = r["d"]
            e["mode%d" % prec] = dd_hex(*r["dd"]) if prec == 0 else r["hex"]
            if prec == 0:                    # the raw double-double, exactly (float.hex)
                e["mode0_dd"] = [r["dd"][0].hex(), r["dd"][1].hex()]
            e["mode%d_seconds" % prec] = r["seconds"]
            e["threads"] = r.get("threads")
            json.dump(data, open(path, "w"), indent=1, sort_keys=True)
            print(p, prec, e, flush=True)


if __name__ == "__main__":
    main()
