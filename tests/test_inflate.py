"""The DEFLATE decoder and CRC-32 the GPU inflates BGZF input with
(fame_gb300/csrc/inflate.h), compiled for the host and checked against zlib
(tests/native/inflate_check.cpp, also under the address and undefined-
behaviour sanitizers); and the tests' BGZF writer against zlib and the
native reader's zlib path (a BGZF file is multi-member gzip)."""
import gzip
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from bgzf_writer import bgzf
from test_fastq import read_all, records

ROOT = Path(__file__).resolve().parents[1]


def build_check(tmp_path, extra):
    exe = tmp_path / "inflate_check"
    subprocess.run(["g++", "-std=c++17", "-I", str(ROOT / "fame_gb300" / "csrc"), *extra,
                    str(ROOT / "tests" / "native" / "inflate_check.cpp"), "-o", str(exe), "-lz"], check=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("flags", [["-O2"], ["-O1", "-g", "-fsanitize=address,undefined"]], ids=["O2", "sanitizers"])
def test_decoder_against_zlib(tmp_path, flags):
    try:
        exe = build_check(tmp_path, flags)
    except subprocess.CalledProcessError:
        if len(flags) > 1:
            pytest.skip("sanitizer runtime not available")
        raise
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert out.startswith("ok "), out
    assert int(out.split()[1]) == 420


def test_bgzf_writer_is_gzip(tmp_path):
    rng = np.random.default_rng(8)
    recs = records(rng, 2000)
    data = b"\n".join(x for r in recs for x in r) + b"\n"
    for level, block in ((0, 65280), (6, 3000), (9, 65280)):
        b = bgzf(data, level, block)
        assert gzip.decompress(b) == data
        p = tmp_path / ("r%d.fq.gz" % level)
        p.write_bytes(b)
        assert read_all(p, True, 700, 3) == [s for _, s, _, _ in recs]   # the zlib path, no device


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_gpu_present(), reason="checks the behaviour without a GPU")
def test_device_paths_fail_loudly_without_a_gpu(tmp_path):
    """With no GPU, BGZF input opened for the device inflater and the device
    index build return FAME_ERR_CUDA (no silent host fallback); plain gzip
    opened with a device still reads through zlib (it never needs one)."""
    from fame_gb300 import FameError, HostIndex
    from fame_gb300._lib import FastqReader
    rng = np.random.default_rng(9)
    recs = records(rng, 500)
    data = b"\n".join(x for r in recs for x in r) + b"\n"
    p = tmp_path / "r.fq.gz"
    p.write_bytes(bgzf(data, 6, 4000))
    with pytest.raises(FameError) as e:
        FastqReader(str(p), is_gz=True, device=0)
    assert e.value.code == -2   # FAME_ERR_CUDA
    q = tmp_path / "plain.fq.gz"
    q.write_bytes(gzip.compress(data))
    r = FastqReader(str(q), is_gz=True, max_reads=1000, max_len=300, device=0)
    assert not r.gpu_inflate
    seq, offs = r.read()
    assert len(offs) - 1 == 500
    r.close()
    with pytest.raises(FameError) as e:
        HostIndex.build_gpu([np.frombuffer(b"ACGT" * 50_000, np.uint8)], readlen=100, device=0)
    assert e.value.code == -2
