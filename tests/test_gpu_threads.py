"""Several contexts on one GPU, one per host thread, running at the same
time (ctypes releases the GIL around library calls): every result equals the
single-threaded one."""
import threading

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_concurrent_contexts(cbl, oracle):
    g = load_golden("oracle_small.json")
    jobs = [(1, 1000000), (1, 10000000), (2, 100000), (1, 10000), (0, 1000000)]
    results, errors = {}, []

    def worker(i, precision, needD):
        try:
            with cbl.Context(0, precision) as ctx:
                for _ in range(3):
                    results[(i, _)] = ctx.compute(needD)
        except Exception as e:                          # reported below, in the main thread
            errors.append((i, repr(e)))

    threads = [threading.Thread(target=worker, args=(i, p, n)) for i, (p, n) in enumerate(jobs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for i, (precision, needD) in enumerate(jobs):
        got = {results[(i, r)] for r in range(3)}
        assert len(got) == 1
        h = got.pop()
        if precision == 0:
            from oracle.oracle import agreeing_hex_digits
            assert agreeing_hex_digits(h, g[str(needD)]["hex256"]) >= 20
        else:
            assert h == g[str(needD)]["hex192"]
