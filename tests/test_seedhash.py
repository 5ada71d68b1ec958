"""The seeding stage's prefix form of the spaced-seed hash
(fame_gb300/csrc/seedhash.h, compiled for the host) against the direct form
over the seed's care positions (NTPS64, spaced_nthash/nthash.hpp), k-mer by
k-mer on random reads of every length up to 255 with ACGT, lower-case, N and
other bytes."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_prefix_hash_matches_direct(tmp_path):
    exe = tmp_path / "seedhash_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "fame_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "seedhash_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "20000"], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok "), out
    assert int(out.split()[1]) > 1_000_000, out
