"""cbl_batch_noalloc, the entry point for callers that may not allocate GPU
memory (for instance a program whose device memory all belongs to its own
allocator or a fixed budget, or a pipeline that must not be stalled by the
synchronisation cudaMalloc/cudaFree can cause). It must give the same 192-bit
results as cbl_batch, call after call, although its scratch array keeps the
previous call's contents. This file is collected last so that a run stopping
at the first failure has already run every other test.
"""
import ctypes
import time

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

CBL_E_LIMIT = -11
MAX_POSITIONS = 64


def _noalloc_fn(cbl):
    L = cbl.load()
    fn = L.cbl_batch_noalloc
    fn.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _call(fn, positions, out, stream):
    arr = (ctypes.c_uint64 * len(positions))(*positions)
    return fn(arr, len(positions), ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))


def _results(out, n):
    w = [int(x) & ((1 << 64) - 1) for x in out[:3 * n].cpu().tolist()]
    return [(w[3 * i] << 128) | (w[3 * i + 1] << 64) | w[3 * i + 2] for i in range(n)]


def test_noalloc_matches_batch_on_consecutive_calls(cbl):
    import torch
    fn = _noalloc_fn(cbl)
    first = [5, 10, 1000, 123455, 10 ** 6, 10 ** 7]
    second = [15, 100, 99995, 10 ** 5, 3 * 10 ** 6, 10 ** 8]
    with cbl.Context(0, 1) as ctx:
        want_first = ctx.batch(first)
        want_second = ctx.batch(second)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    # the caller owns the output buffer; the entry point allocates nothing
    out = torch.full((3 * MAX_POSITIONS,), -1, dtype=torch.int64, device="cuda")
    for positions, want in ((first, want_first), (second, want_second), (first, want_first)):
        out.fill_(-1)
        assert _call(fn, positions, out, stream) == 0
        stream.synchronize()
        assert _results(out, len(positions)) == want


def test_noalloc_limit_and_arguments(cbl):
    import torch
    fn = _noalloc_fn(cbl)
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    out = torch.zeros(3 * (MAX_POSITIONS + 1), dtype=torch.int64, device="cuda")
    too_many = [10 ** 4] * (MAX_POSITIONS + 1)
    assert _call(fn, too_many, out, stream) == CBL_E_LIMIT
    assert _call(fn, [4], out, stream) == -2                 # invalid position
    full = [10 ** 3 + 10 * i for i in range(MAX_POSITIONS)]   # exactly the limit is accepted
    assert _call(fn, full, out, stream) == 0
    stream.synchronize()
    with cbl.Context(0, 1) as ctx:
        assert _results(out, MAX_POSITIONS) == ctx.batch(full)


def test_noalloc_two_word_moduli_and_asynchronous_return(cbl):
    """Position 1e10 runs moduli up to 4e10 (> 2^32, the two-word residue
    kinds). The call only enqueues work: it returns while the GPU is still
    busy (about a second of work), and the result then equals cbl_batch and
    the oracle, on two calls in a row."""
    import torch
    fn = _noalloc_fn(cbl)
    want = int(load_golden("oracle_big.json")["10000000000"]["hex192"], 16)
    with cbl.Context(0, 1) as ctx:
        assert ctx.batch([10 ** 10]) == [want]
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    out = torch.full((3 * MAX_POSITIONS,), -1, dtype=torch.int64, device="cuda")
    for _ in range(2):
        out.fill_(-1)
        stream.synchronize()
        t0 = time.perf_counter()
        assert _call(fn, [10 ** 10, 10 ** 6], out, stream) == 0
        host_s = time.perf_counter() - t0
        still_running = not stream.query()
        stream.synchronize()
        assert _results(out, 2) == [want, int(load_golden("oracle_small.json")["1000000"]["hex192"], 16)]
        assert host_s < 0.1 and still_running
