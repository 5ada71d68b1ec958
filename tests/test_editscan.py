"""The window-scan automaton (fame_gb300/csrc/editscan.h, Myers' bit-vector
recurrence, compiled for the host) against the 7-layer ShiftAnd<6> automaton
(ShiftAnd.h:276-341) restated directly, position by position: read lengths
across every pattern width and its word edges, both read orientations, read N
bases, bisulfite T-to-C text, and N runs that reset both."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_editscan_matches_shiftand(tmp_path):
    exe = tmp_path / "editscan_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "fame_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "editscan_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "20000"], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok 20000 "), out
    assert int(out.split()[2]) > 10_000_000, out
