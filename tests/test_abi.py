"""The C ABI library: it loads, exports every function include/clbellard.h
declares, and its host-only entry points behave like the reference (CPU)."""
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "clbellard.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cbl_\w+)\s*\(", src)))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for n in ("cbl_Sglobal32mtg", "cbl_Sglobal64mtg", "cbl_Sglobal_after", "cbl_Ssum", "cbl_Sum7",
              "cbl_BatchCalc", "cbl_AddAns", "cbl_Set0mem", "cbl_compute", "cbl_run_job",
              "cbl_workmode_sum", "cbl_batch", "cbl_query", "cbl_wait"):
        assert n in names


def test_library_exports_every_declared_symbol(cbl):
    out = subprocess.run(["nm", "-D", "--defined-only", cbl.library_path()], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (cbl_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    lib = cbl.load()
    for n in declared_functions():
        getattr(lib, n)


def test_pos_to_d_matches_oracle(cbl, oracle):
    for p in (5, 7, 10, 12345, 10 ** 8, 10 ** 10, 10 ** 11, 999999999999999999):
        assert cbl.pos_to_d(p) == oracle.pos_to_d(p)
    for p in (0, 4, 10 ** 18):
        with pytest.raises(cbl.CblError) as e:
            cbl.pos_to_d(p)
        assert e.value.code == -2


def test_pointer_variant(cbl):
    import ctypes
    L = cbl.load()
    n, d, a = ctypes.c_int64(10 ** 10), ctypes.c_int64(), ctypes.c_int64()
    assert L.cbl_pos_to_d_p(ctypes.byref(n), ctypes.byref(d), ctypes.byref(a)) == 0
    assert (d.value, a.value) == (3999999999, 10 ** 10)


def test_formula(cbl):
    assert [cbl.formula(f) for f in range(7)] == [
        (32, 1, 4, 1), (1, 1, 4, 3), (256, 0, 10, 1), (64, 1, 10, 3), (4, 1, 10, 5), (4, 1, 10, 7), (1, 0, 10, 9)]
    with pytest.raises(cbl.CblError):
        cbl.formula(7)


def test_workmode_sum_matches_oracle(cbl, oracle):
    import random
    rng = random.Random(3)
    hs = ["%048x" % rng.getrandbits(192) for _ in range(23)]
    assert cbl.workmode_sum(hs) == oracle.hex48_sum(hs) == "%048x" % (sum(int(h, 16) for h in hs) % (1 << 192))
    assert cbl.workmode_sum([]) == "0" * 48
    with pytest.raises(cbl.CblError):
        cbl.workmode_sum(["z" * 48])
    with pytest.raises(cbl.CblError):
        cbl.workmode_sum(["abc"])


def test_strerror(cbl):
    L = cbl.load()
    for code in range(-10, 2):
        assert L.cbl_strerror(code)


def test_no_device_fails_loudly(cbl):
    """No CPU fallback: without a usable GPU, creating a context raises."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(cbl.CblError) as e:
        cbl.Context(0, 1)
    assert e.value.code == -3


def test_tools_fail_loudly_without_gpu(cbl):
    """The profiling entry and the driver exit non-zero with the library's
    no-device error instead of printing nothing or falling back to the CPU."""
    import sys
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from clbellard_gb300 import build
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for args in ([], ["--range", "0", "1000", "2000"]):
        r = subprocess.run([sys.executable, "-m", "clbellard_gb300.profile_case", "--position", "1000000"] + args,
                           cwd=root, capture_output=True, text=True)
        assert r.returncode != 0 and "no CUDA device" in r.stderr
    r = subprocess.run([build.DRIVER, "normal", "1000000"], capture_output=True, text=True)
    assert r.returncode != 0 and "no CUDA device" in r.stderr


def test_driver_binary_built(cbl):
    from clbellard_gb300 import build
    assert os.path.exists(build.DRIVER)
    r = subprocess.run([build.DRIVER], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def test_noalloc_validates_before_touching_the_device(cbl):
    """cbl_batch_noalloc checks its arguments on the host first: too many
    positions is CBL_E_LIMIT and a position outside [5, 999999999999999999] is
    CBL_E_POSITION; the largest valid position passes validation (the kernels
    cover moduli up to 2^62) and only then needs the GPU."""
    import ctypes
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    L = cbl.load()
    fn = L.cbl_batch_noalloc
    fn.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    dummy = ctypes.c_void_p(16)                     # never dereferenced: every call fails before any launch

    def call(pos):
        arr = (ctypes.c_uint64 * len(pos))(*pos)
        return fn(arr, len(pos), dummy, None)

    assert call([10 ** 4] * 65) == -11
    assert call([4]) == -2
    assert call([10 ** 18]) == -2
    assert call([999999999999999999]) in (-3, -5)   # no device / CUDA error, not a position error
    assert fn(None, 0, None, None) == 0
