"""Build libclbellard.so (CUDA, sm_103a) and the `cbl` C driver in-tree.

nvcc compiles the two translation units in parallel and links a shared
library at clbellard_gb300/_build/libclbellard.so; gcc links the driver
clbellard_gb300/_build/cbl against it. No cmake, no torch extension machinery.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libclbellard.so")
DRIVER = os.path.join(OUT, "cbl")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
UNITS = ["cbl_kernels.cu", "cbl_host.cu", "cbl_noalloc.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)]


def _stale(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = _sources() + [os.path.join(INCLUDE, "clbellard.h"), __file__]
    return any(os.path.getmtime(p) > t for p in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    """Compile if any source is newer than the library; return the .so path."""
    if not force and not _stale(LIB) and not _stale(DRIVER):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    flags = NVCC_FLAGS + list(extra_flags or [])
    objs = [os.path.join(OUT, u.replace(".cu", ".o")) for u in UNITS]
    cmds = [[nvcc()] + ARCH + flags + ["-c", os.path.join(CSRC, u), "-o", o] for u, o in zip(UNITS, objs)]
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        outs = list(ex.map(_run, cmds))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    tmp = LIB + ".tmp"
    _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    cc = os.environ.get("CC", "gcc")
    _run([cc, "-O2", "-Wall", "-I", INCLUDE, os.path.join(CSRC, "cbl_main.c"), "-o", DRIVER + ".tmp",
          "-L", OUT, "-lclbellard", "-Wl,-rpath,$ORIGIN"])
    os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


def ptxas_report() -> str:
    """Register / spill / shared-memory report of the kernels (-Xptxas -v)."""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-Xptxas", "-v", "-c", os.path.join(CSRC, "cbl_kernels.cu"),
                                          "-o", os.path.join(OUT, "ptxas_probe.o")]
    os.makedirs(OUT, exist_ok=True)
    return _run(cmd)


if __name__ == "__main__":
    if "--ptxas" in sys.argv:
        print(ptxas_report())
    else:
        print(build(force="--force" in sys.argv, verbose=True))
