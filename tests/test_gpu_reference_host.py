"""The drop-in on FAME's own host: FAME's command-line program (its main.cpp,
parseChunk, decideStrand, index loader and report writer) built with the
bodies of ReadQueue::matchReads and ReadQueue::matchPairedReads replaced by
calls into libfame_gpu.so (tests/reference_host/make_gpu_fame.py), against
the same program built from the unmodified sources.

Both load the index the reference itself built and stored (FAME --genome ...
--store_index ...) and run `--load_index idx -r reads.fq -o out` (and the
paired form, `-r1 -r2`); the CpG reports (<out>_cpg.tsv, main.cpp:363-441,
ReadQueue.cpp:1860-1893) must be equal byte for byte, as must the matching
summary lines FAME prints."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "reference_host"))


@pytest.fixture(scope="module")
def fame(tmp_path_factory, golden):
    import make_gpu_fame
    if not os.path.exists(os.path.join(make_gpu_fame.SRC, "main.cpp")):
        pytest.skip("reference sources not staged (oracle/build_ref.sh)")
    exes = make_gpu_fame.build()
    d = tmp_path_factory.mktemp("fame_host")
    fa = d / "genome.fa"
    lens = golden["chrom_lens"]
    g = golden["genome"]
    with open(fa, "wb") as f:
        o = 0
        for i, L in enumerate(lens):
            f.write(b">chr%d\n" % (i + 1))
            s = g[o:o + L].tobytes()
            for k in range(0, len(s), 80):
                f.write(s[k:k + 80] + b"\n")
            o += L
    idx = d / "genome.idx"
    subprocess.run([exes["stock"], "--genome", str(fa), "--store_index", str(idx)], check=True, cwd=d,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return exes, d, idx


def write_fastq(path, seq, offs):
    with open(path, "wb") as f:
        for i in range(len(offs) - 1):
            r = seq[int(offs[i]):int(offs[i + 1])]
            f.write(b"@r%d\n%s\n+\n%s\n" % (i, r, b"I" * len(r)))


def run(exe, d, args, tag):
    out = d / tag
    p = subprocess.run([exe] + args + ["-o", str(out)], cwd=d, capture_output=True, text=True, check=True)
    # the matching summary FAME prints (counts of matched / non-unique / unmatched reads)
    summary = [ln for ln in p.stdout.splitlines() if re.search(r"(?i)match|pair|read", ln) and re.search(r"\d", ln)
               and "second" not in ln.lower() and " in " not in ln]
    return open(str(out) + "_cpg.tsv", "rb").read(), summary


def test_single_end_cli(fame, golden):
    exes, d, idx = fame
    fq = d / "reads.fq"
    write_fastq(fq, golden["read_seq"].tobytes(), golden["read_offs"])
    args = ["--load_index", str(idx), "-r", str(fq)]
    stock, s_sum = run(exes["stock"], d, args, "stock_se")
    gpu, g_sum = run(exes["gpu"], d, args, "gpu_se")
    assert len(stock) > 10_000
    assert gpu == stock
    assert g_sum == s_sum


def test_paired_end_cli(fame, pe_golden):
    if int(pe_golden["maxpdist"]) != 550:
        pytest.skip("fixture made with another MAXPDIST")
    exes, d, idx = fame
    f1, f2 = d / "r1.fq", d / "r2.fq"
    write_fastq(f1, pe_golden["read_seq1"].tobytes(), pe_golden["read_offs1"])
    write_fastq(f2, pe_golden["read_seq2"].tobytes(), pe_golden["read_offs2"])
    args = ["--load_index", str(idx), "-r1", str(f1), "-r2", str(f2)]
    stock, s_sum = run(exes["stock"], d, args, "stock_pe")
    gpu, g_sum = run(exes["gpu"], d, args, "gpu_pe")
    assert len(stock) > 10_000
    assert gpu == stock
    assert g_sum == s_sum
