"""GB300 Bellard pi hex-digit library: Python host side over libclbellard.so.

The compute path is the CUDA library built from clbellard_gb300/csrc (see
build.py); this module only binds its C ABI (include/clbellard.h) with ctypes
and mirrors the reference's host-side names (KernelFuncs.as: Set0mem,
BatchCalc, AddAns; Bellard.cl kernels: Sglobal32mtg, Sglobal64mtg,
Sglobal_after, Ssum, Sum7). There is no CPU fallback: if the library cannot
be loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

__all__ = ["Context", "CblError", "load", "pos_to_d", "workmode_sum", "formula", "library_path", "plan_jobs",
           "BATCHSIZE", "SKIPPED"]

BATCHSIZE = 137438953472          # 2^37 k-values per work-mode job (Bellard_192.hsp:19)
SKIPPED = 1

_lib = None


class CblError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = _lib.cbl_strerror(code).decode() if _lib is not None else str(code)
        super().__init__("%s: %s (%d)" % (what, msg, code) if what else "%s (%d)" % (msg, code))


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libclbellard.so (building it first if asked and needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libclbellard.so is not built (run clbellard_gb300/build.py)")
    L = ctypes.CDLL(path)
    u64, i64, c_int, vp = ctypes.c_uint64, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
    P64 = ctypes.POINTER(ctypes.c_uint64)
    sigs = {
        "cbl_create": ([c_int, c_int, ctypes.POINTER(vp)], c_int),
        "cbl_destroy": ([vp], c_int),
        "cbl_precision": ([vp], c_int),
        "cbl_stream": ([vp], vp),
        "cbl_device_name": ([vp, ctypes.c_char_p, c_int], c_int),
        "cbl_Set0mem": ([vp], c_int),
        "cbl_Set0ans": ([vp], c_int),
        "cbl_Sglobal32mtg": ([vp, u64, u64, u64, i64, u64, u64], c_int),
        "cbl_Sglobal64mtg": ([vp, u64, u64, u64, i64, u64, u64], c_int),
        "cbl_Sglobal_after": ([vp, u64, i64, u64, u64], c_int),
        "cbl_Ssum": ([vp], c_int),
        "cbl_Sum7": ([vp, u64], c_int),
        "cbl_formula": ([c_int, P64, ctypes.POINTER(i64), P64, P64], c_int),
        "cbl_BatchCalc": ([vp, u64, u64, c_int, u64], c_int),
        "cbl_AddAns": ([vp, c_int], c_int),
        "cbl_read_partial": ([vp, vp], c_int),
        "cbl_read_ans": ([vp, vp], c_int),
        "cbl_query": ([vp], c_int),
        "cbl_wait": ([vp, c_int], c_int),
        "cbl_pos_to_d": ([u64, P64, P64], c_int),
        "cbl_compute": ([vp, u64, ctypes.c_char_p], c_int),
        "cbl_compute_hexpos": ([vp, u64, ctypes.c_char_p], c_int),
        "cbl_run_job": ([vp, u64, c_int, u64, u64, ctypes.c_char_p], c_int),
        "cbl_run_job_range": ([vp, u64, c_int, u64, u64, ctypes.c_char_p], c_int),
        "cbl_plan_jobs": ([u64, c_int, ctypes.POINTER(c_int), P64, P64, c_int], c_int),
        "cbl_workmode_sum": ([ctypes.POINTER(ctypes.c_char_p), c_int, ctypes.c_char_p], c_int),
        "cbl_job_write": ([ctypes.c_char_p, c_int, u64, ctypes.c_char_p, c_int, ctypes.c_char_p, i64], c_int),
        "cbl_job_read": ([ctypes.c_char_p, c_int, u64, ctypes.c_char_p], c_int),
        "cbl_workdir_sum": ([ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(c_int)], c_int),
        "cbl_batch": ([vp, P64, c_int, P64], c_int),
        "cbl_terms": ([vp, u64, c_int, P64, c_int, P64], c_int),
        "cbl_launch_count": ([vp], i64),
        "cbl_prepare": ([vp, P64, c_int], c_int),
        "cbl_run_prepared": ([vp], c_int),
        "cbl_kernel_ms": ([vp, ctypes.POINTER(ctypes.c_float)], c_int),
        "cbl_run_prepared_budget": ([vp, ctypes.c_double, P64, P64], c_int),
        "cbl_checkpoint_size": ([vp], i64),
        "cbl_checkpoint_save": ([vp, vp, i64], c_int),
        "cbl_checkpoint_load": ([vp, vp, i64], c_int),
        "cbl_set_graph": ([vp, c_int], c_int),
        "cbl_autotune": ([vp, P64, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                          ctypes.POINTER(ctypes.c_double)], c_int),
        "cbl_read_results": ([vp, P64], c_int),
        "cbl_prepared_info": ([vp, P64, P64, ctypes.POINTER(c_int), ctypes.POINTER(c_int)], c_int),
        "cbl_probe_imad": ([vp, c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)], c_int),
        "cbl_set_tuning": ([vp, c_int, c_int], c_int),
        "cbl_set_slot_preset": ([vp, P64], c_int),
        "cbl_hex_dd": ([ctypes.c_double, ctypes.c_double, ctypes.c_char_p], c_int),
        "cbl_strerror": ([c_int], ctypes.c_char_p),
        "cbl_pos_to_d_p": ([ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(i64)], c_int),
        "cbl_compute_p": ([vp, ctypes.POINTER(i64), ctypes.c_char_p], c_int),
        "cbl_BatchCalc_p": ([vp, ctypes.POINTER(i64), ctypes.POINTER(i64), c_int, ctypes.POINTER(i64)], c_int),
        "cbl_run_job_p": ([vp, ctypes.POINTER(i64), c_int, ctypes.POINTER(i64), ctypes.POINTER(i64),
                           ctypes.c_char_p], c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise CblError(rc, what)
    return rc


def pos_to_d(needD: int):
    """(d, adjusted needD) for a reference position, as Bellard_192.hsp:468-470."""
    L = load()
    d, a = ctypes.c_uint64(), ctypes.c_uint64()
    _check(L.cbl_pos_to_d(needD, ctypes.byref(d), ctypes.byref(a)), "cbl_pos_to_d")
    return d.value, a.value


def formula(f: int):
    """(numer, numesign, den0, den1) of series f (KernelFuncs.as:9-12)."""
    L = load()
    n, s, a, b = ctypes.c_uint64(), ctypes.c_int64(), ctypes.c_uint64(), ctypes.c_uint64()
    _check(L.cbl_formula(f, ctypes.byref(n), ctypes.byref(s), ctypes.byref(a), ctypes.byref(b)), "cbl_formula")
    return n.value, s.value, a.value, b.value


def workmode_sum(hexes) -> str:
    """workmodeSum0_6: sum of 48-digit hex strings mod 16^48."""
    L = load()
    arr = (ctypes.c_char_p * max(1, len(hexes)))(*[h.encode() for h in hexes])
    out = ctypes.create_string_buffer(49)
    _check(L.cbl_workmode_sum(arr, len(hexes), out), "cbl_workmode_sum")
    return out.value.decode()


def plan_jobs(needD: int, njobs: int):
    """Balanced work-mode jobs: [(s, k0, k1)] of about equal estimated cost."""
    L = load()
    S = (ctypes.c_int * njobs)()
    K0 = (ctypes.c_uint64 * njobs)()
    K1 = (ctypes.c_uint64 * njobs)()
    n = _check(L.cbl_plan_jobs(needD, njobs, S, K0, K1, njobs), "cbl_plan_jobs")
    return [(S[i], K0[i], K1[i]) for i in range(n)]


def hex_dd(hi: float, lo: float) -> str:
    """Mode-0 print form of a double-double (cbl_hex_dd)."""
    out = ctypes.create_string_buffer(49)
    _check(load().cbl_hex_dd(hi, lo, out), "cbl_hex_dd")
    return out.value.decode()


def words_to_int(w) -> int:
    """uint64[3], most significant first -> int."""
    return (int(w[0]) << 128) | (int(w[1]) << 64) | int(w[2])


class Context:
    """One device context: the reference's device buffers bigSum / smallSum /
    dev_ans, a CUDA stream and the kernel entry points."""

    def __init__(self, device: int = 0, precision: int = 1):
        L = load()
        h = ctypes.c_void_p()
        _check(L.cbl_create(device, precision, ctypes.byref(h)), "cbl_create")
        self._h = h
        self.device = device
        self.precision = precision

    # -- lifetime
    def close(self):
        if self._h:
            load().cbl_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return load().cbl_stream(self._h) or 0

    @property
    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        _check(load().cbl_device_name(self._h, buf, 256), "cbl_device_name")
        return buf.value.decode()

    @property
    def launch_count(self) -> int:
        return load().cbl_launch_count(self._h)

    def set_tuning(self, tile_terms: int, ctas_per_sm: int = 0):
        _check(load().cbl_set_tuning(self._h, tile_terms, ctas_per_sm), "cbl_set_tuning")

    # -- reference kernel entry points
    def Set0mem(self):
        _check(load().cbl_Set0mem(self._h), "Set0mem")

    def Set0ans(self):
        _check(load().cbl_Set0ans(self._h), "Set0ans")

    def Sglobal32mtg(self, offset, d, k_max, numesign, den0, den1):
        _check(load().cbl_Sglobal32mtg(self._h, offset, d, k_max, numesign, den0, den1), "Sglobal32mtg")

    def Sglobal64mtg(self, offset, d, k_max, numesign, den0, den1):
        _check(load().cbl_Sglobal64mtg(self._h, offset, d, k_max, numesign, den0, den1), "Sglobal64mtg")

    def Sglobal_after(self, d, numesign, den0, den1):
        _check(load().cbl_Sglobal_after(self._h, d, numesign, den0, den1), "Sglobal_after")

    def Ssum(self):
        _check(load().cbl_Ssum(self._h), "Ssum")

    def Sum7(self, numer: int):
        _check(load().cbl_Sum7(self._h, numer), "Sum7")

    def BatchCalc(self, k_start: int, k_end: int, formulano: int, d: int):
        _check(load().cbl_BatchCalc(self._h, k_start, k_end, formulano, d), "BatchCalc")

    def AddAns(self, formulano: int):
        _check(load().cbl_AddAns(self._h, formulano), "AddAns")

    def _read(self, fn):
        if self.precision == 0:
            buf = (ctypes.c_double * 2)()
            _check(fn(self._h, buf), "read")
            return (buf[0], buf[1])
        buf = (ctypes.c_uint64 * 3)()
        _check(fn(self._h, buf), "read")
        return words_to_int(buf)

    def read_partial(self):
        """int (192-bit, modes 1-2) or (hi, lo) (mode 0)."""
        return self._read(load().cbl_read_partial)

    def read_ans(self):
        return self._read(load().cbl_read_ans)

    def query(self) -> int:
        return _check(load().cbl_query(self._h), "query")

    def wait(self, timeout_ms: int = -1):
        _check(load().cbl_wait(self._h, timeout_ms), "wait")

    # -- application level
    def compute(self, needD: int) -> str:
        out = ctypes.create_string_buffer(49)
        _check(load().cbl_compute(self._h, needD, out), "compute")
        return out.value.decode()

    def compute_hexpos(self, p: int) -> str:
        out = ctypes.create_string_buffer(49)
        _check(load().cbl_compute_hexpos(self._h, p, out), "compute_hexpos")
        return out.value.decode()

    def run_job(self, needD: int, s: int, b: int, batchsize: int = BATCHSIZE):
        """Hex of job (s, b), or None when the reference would skip it."""
        out = ctypes.create_string_buffer(49)
        rc = _check(load().cbl_run_job(self._h, needD, s, b, batchsize, out), "run_job")
        return None if rc == SKIPPED else out.value.decode()

    def run_job_range(self, needD: int, s: int, k0: int, k1: int):
        """Hex of a job over k in [k0, k1) of series s, or None if k0 > d."""
        out = ctypes.create_string_buffer(49)
        rc = _check(load().cbl_run_job_range(self._h, needD, s, k0, k1, out), "run_job_range")
        return None if rc == SKIPPED else out.value.decode()

    def batch(self, positions):
        """192-bit results (ints) for many reference positions in one launch."""
        n = len(positions)
        pos = (ctypes.c_uint64 * max(1, n))(*positions)
        out = (ctypes.c_uint64 * max(3, 3 * n))()
        _check(load().cbl_batch(self._h, pos, n, out), "batch")
        return [words_to_int(out[3 * i:3 * i + 3]) for i in range(n)]

    # -- prepared runs (benchmarks)
    def prepare(self, positions):
        n = len(positions)
        pos = (ctypes.c_uint64 * max(1, n))(*positions)
        _check(load().cbl_prepare(self._h, pos, n), "prepare")
        self._prepared = n

    def run_prepared(self):
        _check(load().cbl_run_prepared(self._h), "run_prepared")

    def run_prepared_budget(self, budget_ms: float):
        """Run or continue a pass for about budget_ms; (tiles_done, tiles_total)."""
        done, total = ctypes.c_uint64(), ctypes.c_uint64()
        _check(load().cbl_run_prepared_budget(self._h, budget_ms, ctypes.byref(done), ctypes.byref(total)),
               "run_prepared_budget")
        return done.value, total.value

    def checkpoint(self) -> bytes:
        n = _check(load().cbl_checkpoint_size(self._h), "checkpoint_size")
        buf = ctypes.create_string_buffer(n)
        _check(load().cbl_checkpoint_save(self._h, buf, n), "checkpoint_save")
        return buf.raw

    def restore(self, blob: bytes):
        buf = ctypes.create_string_buffer(blob, len(blob))
        _check(load().cbl_checkpoint_load(self._h, buf, len(blob)), "checkpoint_load")

    def autotune(self, positions, force: bool = False):
        """Pick tile size and CTAs/SM for these positions (cached); (tile, ctas, ms)."""
        n = len(positions)
        pos = (ctypes.c_uint64 * n)(*positions)
        t, c, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(load().cbl_autotune(self._h, pos, n, 1 if force else 0, ctypes.byref(t), ctypes.byref(c),
                                   ctypes.byref(ms)), "autotune")
        self._prepared = n
        return t.value, c.value, ms.value

    def set_slot_preset(self, preset=None):
        """Test hook: the six digit sums every slot of later prepared passes
        starts from (None = zero); see cbl_set_slot_preset."""
        arr = None if preset is None else (ctypes.c_uint64 * 6)(*[int(x) & (2 ** 64 - 1) for x in preset])
        _check(load().cbl_set_slot_preset(self._h, arr), "cbl_set_slot_preset")

    def set_graph(self, enable: bool):
        _check(load().cbl_set_graph(self._h, 1 if enable else 0), "set_graph")

    def kernel_ms(self) -> float:
        """Device time (CUDA events) of the term kernel in the last run_prepared."""
        ms = ctypes.c_float()
        _check(load().cbl_kernel_ms(self._h, ctypes.byref(ms)), "kernel_ms")
        return ms.value

    def read_results(self):
        n = getattr(self, "_prepared", 0)
        out = (ctypes.c_uint64 * max(3, 3 * n))()
        _check(load().cbl_read_results(self._h, out), "read_results")
        return [words_to_int(out[3 * i:3 * i + 3]) for i in range(n)]

    def prepared_info(self):
        t, n = ctypes.c_uint64(), ctypes.c_uint64()
        s, g = ctypes.c_int(), ctypes.c_int()
        _check(load().cbl_prepared_info(self._h, ctypes.byref(t), ctypes.byref(n), ctypes.byref(s),
                                        ctypes.byref(g)), "prepared_info")
        return {"terms": t.value, "tiles": n.value, "segments": s.value, "grid": g.value}

    def probe_imad(self, iters: int = 4096):
        """(multiply halves per second, ms) of the IMAD throughput probe."""
        ops, ms = ctypes.c_double(), ctypes.c_double()
        _check(load().cbl_probe_imad(self._h, iters, ctypes.byref(ops), ctypes.byref(ms)), "probe_imad")
        return ops.value, ms.value

    def terms(self, d: int, f: int, ks):
        """Signed 192-bit terms (ints) of series f at position d for each k."""
        n = len(ks)
        karr = (ctypes.c_uint64 * max(1, n))(*ks)
        out = (ctypes.c_uint64 * max(3, 3 * n))()
        _check(load().cbl_terms(self._h, d, f, karr, n, out), "terms")
        return [words_to_int(out[3 * i:3 * i + 3]) for i in range(n)]
