"""Run one reference position through the prepared path twice (warm-up + one
measured pass) and print the result and the term-kernel time. Small enough to
run under a profiler:

    python -m clbellard_gb300.profile_case --position 1000000000
"""
from __future__ import annotations

import argparse

import clbellard_gb300 as C


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--position", type=int, default=10 ** 9)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--tile", type=int, default=0)
    ap.add_argument("--ctas", type=int, default=0)
    args = ap.parse_args()
    with C.Context(args.device, 1) as ctx:
        if args.tile:
            ctx.set_tuning(args.tile, args.ctas)
        ctx.prepare([args.position])
        ctx.run_prepared()
        ctx.wait()
        ctx.run_prepared()
        ctx.wait()
        print("%048x %.3f ms" % (ctx.read_results()[0], ctx.kernel_ms()))


if __name__ == "__main__":
    main()
