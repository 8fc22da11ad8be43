"""The pointer-taking `_p` entry points an HSP `#uselib` binding calls (HSP
passes 64-bit integers only by variable address): each equals its by-value
form bit for bit, and negative or missing arguments are rejected."""
import ctypes

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

I64P = ctypes.POINTER(ctypes.c_int64)
E_ARG = -1                       # CBL_E_ARG, include/clbellard.h


def lib():
    import clbellard_gb300 as C
    L = C.load()
    L.cbl_compute_p.argtypes = [ctypes.c_void_p, I64P, ctypes.c_char_p]
    L.cbl_BatchCalc_p.argtypes = [ctypes.c_void_p, I64P, I64P, ctypes.c_int, I64P]
    L.cbl_run_job_p.argtypes = [ctypes.c_void_p, I64P, ctypes.c_int, I64P, I64P, ctypes.c_char_p]
    L.cbl_pos_to_d_p.argtypes = [I64P, I64P, I64P]
    for f in ("cbl_compute_p", "cbl_BatchCalc_p", "cbl_run_job_p", "cbl_pos_to_d_p"):
        getattr(L, f).restype = ctypes.c_int
    return L


def i64(v):
    return ctypes.byref(ctypes.c_int64(v))


def test_compute_p(ctx192, cbl):
    L = lib()
    out = ctypes.create_string_buffer(49)
    assert L.cbl_compute_p(ctx192._h, i64(1000000), out) == 0
    assert out.value.decode() == ctx192.compute(1000000) == load_golden("oracle_small.json")["1000000"]["hex192"]
    assert L.cbl_compute_p(ctx192._h, i64(-5), out) == E_ARG
    assert L.cbl_compute_p(ctx192._h, None, out) == E_ARG


def test_pos_to_d_p(cbl):
    L = lib()
    d, adj = ctypes.c_int64(), ctypes.c_int64()
    assert L.cbl_pos_to_d_p(i64(10 ** 10), ctypes.byref(d), ctypes.byref(adj)) == 0
    assert (d.value, adj.value) == (3999999999, 10 ** 10)
    assert L.cbl_pos_to_d_p(i64(-1), ctypes.byref(d), ctypes.byref(adj)) == E_ARG


def test_batchcalc_p_equals_by_value(ctx192, cbl, oracle):
    """Set0mem, BatchCalc_p over a range, AddAns: the reference's per-series call order."""
    L = lib()
    needD = 100000
    d, _ = oracle.pos_to_d(needD)
    got = []
    for s, k0, k1 in [(0, 0, 17), (3, 1000, 5000), (6, 35000, d + 20)]:
        ctx192.Set0mem()
        assert L.cbl_BatchCalc_p(ctx192._h, i64(k0), i64(k1), s, i64(d)) == 0
        ctx192.AddAns(s)
        got.append(ctx192.read_partial())
        assert got[-1] == int(ctx192.run_job_range(needD, s, k0, k1), 16)
    assert L.cbl_BatchCalc_p(ctx192._h, i64(-1), i64(5), 0, i64(d)) == E_ARG
    assert L.cbl_BatchCalc_p(ctx192._h, i64(0), i64(5), 7, i64(d)) == E_ARG


def test_run_job_p_equals_by_value(ctx192, cbl):
    L = lib()
    out = ctypes.create_string_buffer(49)
    for s in range(7):
        assert L.cbl_run_job_p(ctx192._h, i64(100000), s, i64(1), i64(7919), out) == 0
        assert out.value.decode() == ctx192.run_job(100000, s, 1, 7919)
    # a batch that starts past d is skipped, as the reference skips it
    assert L.cbl_run_job_p(ctx192._h, i64(100000), 0, i64(10 ** 6), i64(7919), out) == cbl.SKIPPED
    assert L.cbl_run_job_p(ctx192._h, i64(100000), 0, i64(0), i64(0), out) == E_ARG
