"""The Shift-And pre-filter's q-gram pass (fame_gb300/csrc/qgram.h, compiled
for the host) against the direct scan-order formulation, on random windows of
both scan directions with N runs, window edges inside packed words and
low-complexity text (span overflow and fallback)."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_qgram_spans_match_scan_order(tmp_path):
    exe = tmp_path / "qgram_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "fame_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "qgram_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "20000"], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok 20000 cases"), out
