"""Compile the reference's own kernels (Bellard.cl, Bellard_div2by1.cl) as
C++ for the CPU into oracle/_ref/ref_bellard, and a second time with
-DOVERDOUBLE into oracle/_ref/ref_bellard_od (the build the reference's host
selects when a modulus can reach 2^53, Bellard_192.hsp:472).

TEST INFRASTRUCTURE: the reference run here pins the oracle and gives a CPU
baseline. The sources are read from the reference tree where they lie; a
temporary copy outside this repository receives one textual rewrite (an
in-kernel `__local T p[...]` work-group array becomes `static thread_local`, so
the fibers of one work-group share it) and is deleted after the build. Only
the binary is written into oracle/_ref/ (git-ignored).
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT_DIR = os.path.join(ORACLE, "_ref")
BINARY = os.path.join(OUT_DIR, "ref_bellard")
BINARY_OD = os.path.join(OUT_DIR, "ref_bellard_od")
# The reference tree is read where it lies; CBL_REFERENCE_DIR overrides the default location.
REFERENCE = os.environ.get("CBL_REFERENCE_DIR", "/root/reference")
SOURCES = ("Bellard.cl", "Bellard_div2by1.cl")
LOCAL_ARRAY = re.compile(r"^(\s*)__local(\s+\w+\s+\w+\s*\[)", re.M)


def available() -> bool:
    return all(os.path.exists(os.path.join(REFERENCE, s)) for s in SOURCES)


def build_if_available(force: bool = False):
    """Build oracle/_ref/ref_bellard when the reference tree is present.
    Returns the binary path, or None when the reference is absent."""
    if not available():
        return BINARY if os.path.exists(BINARY) else None
    deps = [os.path.join(HERE, "harness.cpp"), os.path.join(HERE, "shim.h"), __file__]
    if not force and all(os.path.exists(b) and all(os.path.getmtime(p) < os.path.getmtime(b) for p in deps)
                         for b in (BINARY, BINARY_OD)):
        return BINARY
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="cbl_ref_")
    try:
        for s in SOURCES:
            text = open(os.path.join(REFERENCE, s), encoding="utf-8").read()
            open(os.path.join(tmp, s), "w", encoding="utf-8").write(LOCAL_ARRAY.sub(r"\1static thread_local\2", text))
        for out, extra in ((BINARY, []), (BINARY_OD, ["-DOVERDOUBLE"])):
            cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-w", *extra,
                   "-I", tmp, "-I", HERE, os.path.join(HERE, "harness.cpp"), "-o", out + ".tmp"]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            if r.returncode != 0:
                raise RuntimeError("reference harness build failed:\n" + r.stdout[-4000:])
            os.replace(out + ".tmp", out)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return BINARY


def runnable() -> bool:
    """True when a reference binary built for this machine exists."""
    b = build_if_available()
    if b is None:
        return False
    try:
        subprocess.run([b], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=30)
    except (OSError, subprocess.SubprocessError):
        return False
    return True


def run(needD: int, precision: int, groups: int = 64, threads: int = 0, timeout: float = 3600.0,
        sample=None) -> dict:
    """Run the reference at one position; returns d, hex (modes 1-2) or (hi, lo)
    (mode 0), seconds and terms/s. sample = (chunk_terms, chunks) times that
    many k-ranges per series spread over [0, d) instead of the full position."""
    b = build_if_available()
    if b is None:
        raise RuntimeError("reference harness not built and the reference tree is absent")
    args = [b, str(needD), str(precision), str(groups), str(threads)]
    if sample:
        args += ["0", str(sample[0]), str(sample[1])]
    out = subprocess.run(args, stdout=subprocess.PIPE, text=True, timeout=timeout, check=True).stdout
    res = {}
    for ln in out.splitlines():
        k, _, v = ln.partition(" ")
        if k == "d":
            res["d"] = int(v)
        elif k == "hex":
            res["hex"] = v.strip()
        elif k == "dd":
            hi, lo = v.split()
            res["dd"] = (float(hi), float(lo))
        elif k == "seconds":
            res["seconds"] = float(v)
        elif k == "terms_per_s":
            res["terms_per_s"] = float(v)
        elif k == "threads":
            res["threads"] = int(v)
    return res


def run_range(needD: int, precision: int, f: int, k0: int, k1: int, groups: int = 64, threads: int = 0,
              timeout: float = 600.0) -> dict:
    """The reference's BatchCalc for series f over k in [k0, min(k1, d)) (plus
    the tail when the range reaches d), after Ssum and before Sum7: returns d
    and the partial as an int (modes 1-2, bigSum[0..2]) or (hi, lo) (mode 0).
    Uses the OVERDOUBLE build when the reference's host would
    (d*10+9 >= 2^53, Bellard_192.hsp:472)."""
    if build_if_available() is None:
        raise RuntimeError("reference harness not built and the reference tree is absent")
    d = ((needD - 1) * 2 - 3) // 5
    if d % 2 == 0:
        d -= 1
    b = BINARY_OD if d * 10 + 9 >= (1 << 53) else BINARY
    args = [b, "range", str(needD), str(precision), str(f), str(k0), str(k1), str(groups), str(threads)]
    out = subprocess.run(args, stdout=subprocess.PIPE, text=True, timeout=timeout, check=True).stdout
    res = {"overdouble": b == BINARY_OD}
    for ln in out.splitlines():
        k, _, v = ln.partition(" ")
        if k == "d":
            res["d"] = int(v)
        elif k == "partial":
            res["partial"] = int(v, 16)
        elif k == "partial_dd":
            hi, lo = v.split()
            res["partial"] = (float(hi), float(lo))
    return res


if __name__ == "__main__":
    print(build_if_available(force="--force" in sys.argv))
