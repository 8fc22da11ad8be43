"""The `cbl` C driver (the CLBellard.exe / workmodeSum0_6.exe roles): normal
mode, work mode with the reference's worklist and job files, and the merge."""
import os
import subprocess

import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def driver():
    from clbellard_gb300 import build
    return build.DRIVER


def test_normal_mode():
    out = subprocess.run([driver(), "normal", "1000000", "1"], capture_output=True, text=True, check=True).stdout
    assert load_golden("oracle_small.json")["1000000"]["hex192"] in out
    assert "loopnum=399999" in out


def test_normal_mode_json_and_overlap_check():
    """One JSON line per run; --check recomputes position P-8 and counts the
    agreeing overlap digits (no oracle in the product)."""
    import json
    out = subprocess.run([driver(), "normal", "10000000", "1", "--json", "--check"], capture_output=True, text=True,
                         check=True).stdout
    rec = json.loads(out.strip().splitlines()[-1])
    assert rec["hex"] == load_golden("oracle_small.json")["10000000"]["hex192"]
    assert rec["position"] == 10000000 and rec["d"] == 3999999 and rec["terms"] == 7 * 3999999
    assert rec["overlap_digits"] >= 28 and rec["terms_per_s"] > 0


def test_work_mode_and_merge(tmp_path):
    wl = tmp_path / "worklist.txt"
    # the reference's worklist layout (work/worklist_sample.txt), CR LF line ends
    wl.write_bytes(b"digits=100000\r\nprecision=1 (0=106bit , 1=192bit)\r\n" +
                   b"".join(b"%d_0\r\n" % s for s in range(7)))
    work = tmp_path / "work"
    r = subprocess.run([driver(), "work", str(wl), str(work)], capture_output=True, text=True, check=True)
    assert r.stdout.strip().endswith("end")
    for s in range(7):
        assert (work / str(s) / ("%d_0.txt" % s)).exists()
    # a second run finds every job done and writes nothing new
    mtimes = [os.path.getmtime(work / str(s) / ("%d_0.txt" % s)) for s in range(7)]
    subprocess.run([driver(), "work", str(wl), str(work)], capture_output=True, text=True, check=True)
    assert mtimes == [os.path.getmtime(work / str(s) / ("%d_0.txt" % s)) for s in range(7)]
    out = subprocess.run([driver(), "sum", str(work)], capture_output=True, text=True, check=True).stdout
    assert load_golden("oracle_small.json")["100000"]["hex192"] in out
    assert "0:1" in out and "6:1" in out


def test_plan_then_work(tmp_path):
    """`cbl plan` writes a balanced worklist that `cbl work` runs and `cbl sum` merges."""
    plan = subprocess.run([driver(), "plan", "1000000", "14"], capture_output=True, text=True, check=True).stdout
    lines = plan.splitlines()
    assert lines[0] == "digits=1000000" and len(lines) == 16
    wl = tmp_path / "worklist.txt"
    wl.write_text(plan)
    work = tmp_path / "work"
    subprocess.run([driver(), "work", str(wl), str(work)], capture_output=True, text=True, check=True)
    out = subprocess.run([driver(), "sum", str(work)], capture_output=True, text=True, check=True).stdout
    assert load_golden("oracle_small.json")["1000000"]["hex192"] in out


def test_hexpos():
    out = subprocess.run([driver(), "hexpos", "5"], capture_output=True, text=True, check=True).stdout
    assert out.startswith("6a8885a308d313198a2e0370734")
