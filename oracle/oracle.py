"""ctypes loader for the exact CPU oracle (oracle/bellard_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the cpu_baseline / reference arm of ``bench.py``, as the checker. The product
library (clbellard_gb300) never imports this module.

Fixed-point values are Python ints in [0, 2^(64W)): floor(x * 2^(64W)) for a
value x taken mod 1 (see bellard_oracle.h for the per-term definition).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

# KernelFuncs.as:9-12
NUMER_LOG2 = (5, 0, 8, 6, 2, 2, 0)
SIGN = (1, 1, 0, 1, 1, 1, 0)
DEN0 = (4, 4, 10, 10, 10, 10, 10)
DEN1 = (1, 3, 1, 3, 5, 7, 9)

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with make (gcc, OpenMP) into oracle/_build/."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "bellard_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64, P64 = ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)
        L.orc_pos_to_d.argtypes = [u64, P64, P64]
        L.orc_hexpos_to_d.argtypes = [u64, P64, ctypes.POINTER(ctypes.c_int)]
        L.orc_pow2mod.argtypes = [u64, u64]
        L.orc_pow2mod.restype = u64
        L.orc_pow2mod_plain.argtypes = [u64, u64]
        L.orc_pow2mod_plain.restype = u64
        L.orc_term.argtypes = [u64, ctypes.c_int, u64, ctypes.c_int, P64]
        L.orc_sum_range.argtypes = [u64, ctypes.c_int, u64, u64, ctypes.c_int, ctypes.c_int, P64]
        L.orc_series.argtypes = [u64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P64]
        L.orc_result.argtypes = [u64, ctypes.c_int, ctypes.c_int, ctypes.c_int, P64]
        L.orc_sum_range34.argtypes = [u64, ctypes.c_int, u64, u64, ctypes.c_int, P64, P64]
        L.orc_result34.argtypes = [u64, ctypes.c_int, ctypes.c_int, P64, P64]
        L.orc_tail_terms.argtypes = [ctypes.c_int]
        L.orc_to_hex.argtypes = [P64, ctypes.c_int, ctypes.c_char_p]
        L.orc_hex48_sum.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.c_char_p]
        L.orc_dd_result.argtypes = [u64, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]
        _lib = L
    return _lib


def _words_to_int(w, W):
    return sum(int(w[i]) << (64 * i) for i in range(W))


def pos_to_d(needD: int):
    """Reference position mapping; returns (d, adjusted needD) or None if invalid."""
    d, a = ctypes.c_uint64(), ctypes.c_uint64()
    if lib().orc_pos_to_d(needD, ctypes.byref(d), ctypes.byref(a)) != 0:
        return None
    return d.value, a.value


def hexpos_to_d(p: int):
    d, s = ctypes.c_uint64(), ctypes.c_int()
    if lib().orc_hexpos_to_d(p, ctypes.byref(d), ctypes.byref(s)) != 0:
        return None
    return d.value, s.value


def pow2mod(e: int, m: int) -> int:
    return lib().orc_pow2mod(e, m)


def pow2mod_plain(e: int, m: int) -> int:
    return lib().orc_pow2mod_plain(e, m)


def term(d: int, f: int, k: int, W: int = 3) -> int:
    out = (ctypes.c_uint64 * W)()
    lib().orc_term(d, f, k, W, out)
    return _words_to_int(out, W)


def sum_range(d: int, f: int, k0: int, k1: int, W: int = 3, nthreads: int = 0) -> int:
    out = (ctypes.c_uint64 * W)()
    lib().orc_sum_range(d, f, k0, k1, W, nthreads, out)
    return _words_to_int(out, W)


def tail_terms(W: int = 3) -> int:
    return lib().orc_tail_terms(W)


def series(d: int, f: int, W: int = 3, nthreads: int = 0) -> int:
    out = (ctypes.c_uint64 * W)()
    lib().orc_series(d, f, W, nthreads, out)
    return _words_to_int(out, W)


def result(d: int, shift: int = 0, W: int = 3, nthreads: int = 0) -> int:
    """frac(2^(10d+6+shift) * pi) as a 64W-bit fixed-point int."""
    out = (ctypes.c_uint64 * W)()
    lib().orc_result(d, shift, W, nthreads, out)
    return _words_to_int(out, W)


def sum_range34(d: int, f: int, k0: int, k1: int, nthreads: int = 0):
    """(W=3 sum, W=4 sum) of series f over [k0, k1) from one pass."""
    o3, o4 = (ctypes.c_uint64 * 3)(), (ctypes.c_uint64 * 4)()
    lib().orc_sum_range34(d, f, k0, k1, nthreads, o3, o4)
    return _words_to_int(o3, 3), _words_to_int(o4, 4)


def result34(d: int, shift: int = 0, nthreads: int = 0):
    """(result(d, shift, 3), result(d, shift, 4)) from one pass over k."""
    o3, o4 = (ctypes.c_uint64 * 3)(), (ctypes.c_uint64 * 4)()
    lib().orc_result34(d, shift, nthreads, o3, o4)
    return _words_to_int(o3, 3), _words_to_int(o4, 4)


def to_hex(x: int, W: int = 3) -> str:
    return format(x, "0%dx" % (16 * W))


def hex48_sum(hexes) -> str | None:
    arr = (ctypes.c_char_p * len(hexes))(*[h.encode() for h in hexes])
    out = ctypes.create_string_buffer(49)
    if lib().orc_hex48_sum(arr, len(hexes), out) != 0:
        return None
    return out.value.decode()


def dd_result(d: int, nthreads: int = 0):
    hi, lo = ctypes.c_double(), ctypes.c_double()
    lib().orc_dd_result(d, nthreads, ctypes.byref(hi), ctypes.byref(lo))
    return hi.value, lo.value


# ---- pure-Python restatement for small cases (independent of the C code) ----
def py_term(d: int, f: int, k: int, W: int = 3) -> int:
    """One signed term with Python big ints: floor(s*x*2^N) mod 2^N."""
    N = 64 * W
    m = DEN0[f] * k + DEN1[f]
    if m == 1:
        return 0
    if k < d:
        q = (pow(2, 10 * (d - k), m) << N) // m
    else:
        i = k - d
        q = (1 << N) // m >> (10 * i) if 10 * i <= N else 0
    if (k + SIGN[f]) & 1:
        q = (~q) & ((1 << N) - 1)
    return q


def py_result(d: int, shift: int = 0, W: int = 3) -> int:
    N = 64 * W
    mask = (1 << N) - 1
    nt = 64 * W // 10 + 1
    acc = 0
    for f in range(7):
        s = 0
        for k in range(d + nt):
            s += py_term(d, f, k, W)
        acc += (s << (NUMER_LOG2[f] + shift))
    return acc & mask


# ---- the reference's mode-0 printer, restated ------------------------------
def _twosum(a: float, b: float):
    """hexsademical.as:3-10."""
    x = a + b
    tmp = x - a
    return x, (a - (x - tmp)) + (b - tmp)


def _addcab(a, b):
    """Double-double add, hexsademical.as:12-19."""
    x, y = _twosum(a[0], b[0])
    y = y + a[1] + b[1]
    return _twosum(x, y)


def _hsp_int(x: float) -> int:
    """HSP int() of a double: truncation toward zero; out of the 32-bit range
    the x86 conversion yields INT_MIN."""
    if x != x or not (-2147483649.0 < x < 2147483648.0):
        return -2147483648
    return int(x)


def hexadecimal_dd(hi: float, lo: float, report: bool = False):
    """The reference's mode-0 result printer, hexadecimal_dd
    (hexsademical.as:21-101, printed by hexadecimal_i32 :104-127), restated
    step by step: a negative value is lifted by 1.0 (:25-31); then 14 times
    the double-double is scaled by 256 and renormalised (:38-44) and its
    integer part becomes the next byte, most significant first, into a
    24-byte little-endian buffer of six 32-bit ints (:46-49). An integer part
    of exactly 256 writes 0 and carries 1 into the byte before, through the
    ints (:51-71); a negative remainder writes int(x + 256) and borrows 1 from
    the byte before (:73-91), then sets the remainder to x + 256 (:92-96), so
    every later byte reads 00. Bytes 9..0 stay 0: 28 hex digits and 20 zeros.
    With report=True returns (hex, whether the borrow branch was taken)."""
    out = bytearray(24)
    borrowed = False

    def get_int(b):
        return int.from_bytes(out[4 * b:4 * b + 4], "little", signed=True)

    def set_int(b, v):
        out[4 * b:4 * b + 4] = (v & 0xffffffff).to_bytes(4, "little")

    def poke(i, v):
        out[i] = v & 0xff

    if hi < 0.0:
        hi, lo = _addcab((hi, lo), (1.0, 0.0))
    for cnt in range(14):
        hi *= 256.0
        lo *= 256.0
        x = hi + lo
        tmp = x - hi
        y = (hi - (x - tmp)) + (lo - tmp)
        hi, lo = x, y
        moji = _hsp_int(hi)
        if moji < 256 and hi >= 0.0:
            poke(23 - cnt, moji)
            hi -= moji
            continue
        if moji == 256:
            moji = moji % 256
            idx = 23 - cnt + 1
            if idx < 24:
                bidx, lidx = idx // 4, idx % 4
                addv = 1 << (lidx * 8)
                set_int(bidx, get_int(bidx) + addv)
                for _ in range(5 - bidx):
                    v = get_int(bidx)
                    if 0 <= v < addv:
                        bidx += 1
                        addv = 1
                        set_int(bidx, get_int(bidx) + addv)
                    else:
                        break
            poke(23 - cnt, moji)
            hi -= 256.0
        if hi < 0.0:
            borrowed = True
            moji = _hsp_int(hi + 256.0)
            idx = 23 - cnt + 1
            if idx < 24:
                bidx, lidx = idx // 4, idx % 4
                addv = 1 << (lidx * 8)
                set_int(bidx, get_int(bidx) - addv)
                for _ in range(5 - bidx):
                    v = get_int(bidx)
                    if -addv <= v < 0:
                        bidx += 1
                        addv = 1
                        set_int(bidx, get_int(bidx) - addv)
                    else:
                        break
            poke(23 - cnt, moji)
            hi, lo = _addcab((hi, lo), (256.0, 0.0))
    h = bytes(reversed(out)).hex()
    return (h, borrowed) if report else h


def dd_exact_hex(hi: float, lo: float, lift: bool = False) -> str:
    """The exact value (hi + lo) mod 1 truncated to 112 bits: 28 hex digits
    and 20 zeros. With lift, a negative hi is first lifted by 1.0 with the
    reference's double-double add (hexsademical.as:25-31), rounding included."""
    from fractions import Fraction
    if lift and hi < 0.0:
        hi, lo = _addcab((hi, lo), (1.0, 0.0))
    v = int((Fraction(hi) + Fraction(lo)) % 1 * (1 << 112))
    return format(v, "028x") + "0" * 20


def agreeing_hex_digits(a: str, b: str) -> int:
    n = 0
    for x, y in zip(a, b):
        if x != y:
            break
        n += 1
    return n
