"""Run one reference position through the prepared path twice (warm-up + one
measured pass) and print the result and the term-kernel time. Small enough to
run under a profiler:

    python -m clbellard_gb300.profile_case --position 1000000000

With --range f k0 k1, run instead one series' BatchCalc over k in [k0, k1)
at the position's d (twice), e.g. a range where one residue kind does all
the work:

    python -m clbellard_gb300.profile_case --position 10000000000 --range 0 3000000000 3100000000

--precision 0 runs that range through the 106-bit double-double kernels instead.
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
    ap.add_argument("--range", type=int, nargs=3, metavar=("F", "K0", "K1"))
    ap.add_argument("--precision", type=int, default=1, choices=[0, 1, 2])
    args = ap.parse_args()
    if args.range:
        import time
        f, k0, k1 = args.range
        d, _ = C.pos_to_d(args.position)
        with C.Context(args.device, args.precision) as ctx:
            if args.tile and args.precision:
                ctx.set_tuning(args.tile, args.ctas)
            for _ in range(2):
                ctx.Set0mem()
                t0 = time.perf_counter()
                ctx.BatchCalc(k0, k1, f, d)
                ctx.wait()
                ms = (time.perf_counter() - t0) * 1e3
            part = ctx.read_partial()
            shown = "%048x" % part if args.precision else "%.17g %.17g" % part
            print("%s %.3f ms (%d terms, wall)" % (shown, ms, k1 - k0))
        return
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
