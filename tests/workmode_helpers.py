"""Job partials computed by the oracle, for the work-mode host tests (the CPU
stands in for the GPUs only in those tests)."""


def oracle_job(oracle, batchsize):
    """The reference's job partial (numer-weighted, 192-bit) for job (s, b)."""
    def fn(needD, s, b, bs):
        return oracle_range(oracle)(needD, s, b * bs, (b + 1) * bs)
    return fn


def oracle_range(oracle):
    """Job partial over an explicit k-range (the tail when the range reaches d)."""
    def fn(needD, s, k0, k1):
        d, _ = oracle.pos_to_d(needD)
        if k0 > d:
            return None
        kend = min(k1, d)
        v = oracle.sum_range(d, s, k0, kend, 3) if k0 < kend else 0
        if max(k0, kend) == d:
            v += oracle.sum_range(d, s, d, d + 20, 3)
        return "%048x" % ((v << oracle.NUMER_LOG2[s]) % (1 << 192))
    return fn
