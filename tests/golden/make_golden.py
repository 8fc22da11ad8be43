"""Generate the oracle golden fixtures in tests/golden/.

    python tests/golden/make_golden.py            # small positions (seconds)
    python tests/golden/make_golden.py --big 100000000000   # 1e11: hours on 8 cores

Each fixture records, for a reference position needD, the oracle's 192-bit
result (the bit-exact definition the CUDA kernels reproduce) and its 256-bit
result (for true-digit agreement). The 256-bit oracle itself is pinned by
published hex digits of pi (Bailey-Borwein-Plouffe positions 10^6 .. 10^11)
and by the reference's own kernels run on the CPU (ref_outputs.json).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

SMALL = [5, 10, 15, 100, 1000, 10000, 100000, 1000000, 10000000]


def entry(needD: int, threads: int) -> dict:
    d, adj = O.pos_to_d(needD)
    t0 = time.time()
    r3, r4 = O.result34(d, 0, threads)      # both widths from one pass over k
    t1 = time.time()
    return {"needD": adj, "d": d, "hex192": O.to_hex(r3, 3), "hex256": O.to_hex(r4, 4),
            "seconds_192_256": round(t1 - t0, 2), "threads": threads or os.cpu_count()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", type=int, nargs="*", default=None)
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    if args.big:
        path = os.path.join(HERE, "oracle_big.json")
        data = json.load(open(path)) if os.path.exists(path) else {}
        for p in args.big:
            data[str(p)] = entry(p, args.threads)
            json.dump(data, open(path, "w"), indent=1, sort_keys=True)
            print(p, data[str(p)], flush=True)
        return
    data = {str(p): entry(p, args.threads) for p in SMALL}
    json.dump(data, open(os.path.join(HERE, "oracle_small.json"), "w"), indent=1, sort_keys=True)
    print(json.dumps(data, indent=1))


if __name__ == "__main__":
    main()
