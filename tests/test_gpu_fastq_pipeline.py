"""fame_match_fastq: a whole FASTQ file parsed and matched overlapped
(queryRoutine, main.cpp:363-399) against the reference's golden chunk loops
and against the chunk-by-chunk host loop (ReadQueue over
fame_gpu_match_reads).  Bit-exact: counters, read count and every CpG tally.
"""
import gzip

import numpy as np
import pytest

from fame_gb300 import FAME_BOTH_STRANDS, FameError, GpuMatcher, ReadQueue

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(product_index):
    g = GpuMatcher(product_index, 0)
    yield g
    g.close()


def write_fastq(path, reads, gz):
    lines = []
    for i, r in enumerate(reads):
        lines += [b"@read%d" % i, r, b"+", b"I" * len(r)]
    with (gzip.open if gz else open)(path, "wb") as f:
        f.write(b"\n".join(lines) + (b"\n" if lines else b""))


def golden_reads(golden, n=None):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    n = len(offs) - 1 if n is None else n
    return [seq[int(offs[i]):int(offs[i + 1])] for i in range(n)]


def counters(c):
    return (c.succ, c.nonunique, c.unsucc, c.r1_fwd, c.r1_rev)


@pytest.mark.parametrize("gz", [False, True], ids=["fastq", "fastq.gz"])
@pytest.mark.parametrize("name,chunk,both,slots", [("default", 0, False, 2), ("chunk1000", 1000, False, 2),
                                                   ("chunk1000", 1000, False, 8), ("both", 777, True, 3)])
def test_match_fastq_golden(gpu, golden, tmp_path, gz, name, chunk, both, slots):
    reads = golden_reads(golden)
    path = tmp_path / ("reads.fq.gz" if gz else "reads.fq")
    write_fastq(path, reads, gz)
    gpu.tallies(reset=True)
    cnt, n = gpu.match_fastq(str(path), gz, FAME_BOTH_STRANDS if both else 0, chunk=chunk, slots=slots)
    c = golden[name + "_counters"]
    assert n == len(reads)
    assert counters(cnt) == tuple(int(x) for x in c[:5])
    assert np.array_equal(gpu.tallies(reset=True), golden[name + "_meth"])


@pytest.mark.parametrize("nreads,chunk,both,slots", [(6000, 1000, False, 2),    # whole chunks: the last parse is empty
                                                     (6000, 1500, True, 4),
                                                     (999, 1000, False, 3),      # one partial chunk
                                                     (1000, 1000, False, 2),     # one full chunk, then an empty one
                                                     (2001, 250, False, 5)])
def test_match_fastq_vs_chunk_loop(gpu, golden, product_index, tmp_path, nreads, chunk, both, slots):
    reads = golden_reads(golden, nreads)
    path = tmp_path / "reads.fq"
    write_fastq(path, reads, False)
    gpu.tallies(reset=True)
    rq = ReadQueue(reads, product_index, gpu, both_strands=both, chunk_size=chunk)
    tot = rq.query_routine()
    exp_meth = gpu.tallies(reset=True)
    cnt, n = gpu.match_fastq(str(path), False, FAME_BOTH_STRANDS if both else 0, chunk=chunk, slots=slots,
                             threads=2)
    assert n == nreads
    assert (cnt.succ, cnt.nonunique, cnt.unsucc) == (tot["succ"], tot["nonunique"], tot["unsucc"])
    assert (cnt.r1_fwd, cnt.r1_rev) == (rq.r1_fwd_matches, rq.r1_rev_matches)
    assert np.array_equal(gpu.tallies(reset=True), exp_meth)


def test_match_fastq_empty_and_errors(gpu, golden, tmp_path):
    empty = tmp_path / "empty.fq"
    write_fastq(empty, [], False)
    gpu.tallies(reset=True)
    cnt, n = gpu.match_fastq(str(empty), False, 0)
    assert n == 0 and counters(cnt) == (0, 0, 0, 0, 0)
    assert not gpu.tallies(reset=True).any()
    with pytest.raises(FameError):
        gpu.match_fastq(str(tmp_path / "missing.fq"), False, 0)
    # a read longer than FAME_MAX_READ_LEN fails the call; the context stays usable
    long_read = tmp_path / "long.fq"
    write_fastq(long_read, golden_reads(golden, 10) + [b"ACGT" * 70], False)
    with pytest.raises(FameError):
        gpu.match_fastq(str(long_read), False, 0, chunk=100)
    gpu.tallies(reset=True)
    ok = tmp_path / "ok.fq"
    write_fastq(ok, golden_reads(golden), False)
    cnt, n = gpu.match_fastq(str(ok), False, 0)
    c = golden["default_counters"]
    assert counters(cnt) == tuple(int(x) for x in c[:5])
    assert np.array_equal(gpu.tallies(reset=True), golden["default_meth"])
