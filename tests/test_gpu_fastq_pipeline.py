"""fame_match_fastq / fame_match_fastq_paired: whole FASTQ files parsed and
matched overlapped (queryRoutine, main.cpp:363-399; queryRoutinePaired,
main.cpp:400-441) against the reference's golden chunk loops and against the
chunk-by-chunk host loops (ReadQueue / PairedReadQueue over
fame_gpu_match_reads / fame_gpu_match_pairs).  Bit-exact: counters, record
counts and every CpG tally.
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


PE_MODES = (("default", 0, False), ("chunk700", 700, False), ("both", 900, True))


def golden_mates(pe_golden):
    out = []
    for k in ("1", "2"):
        s, o = pe_golden["read_seq" + k].tobytes(), pe_golden["read_offs" + k]
        out.append([s[int(o[i]):int(o[i + 1])] for i in range(len(o) - 1)])
    return out


def pair_counters(c):
    return [c.succ, c.nonunique, c.unsucc, c.paired, c.too_short, c.r1_fwd, c.r1_rev]


@pytest.mark.parametrize("gz", [False, True], ids=["fastq", "fastq.gz"])
@pytest.mark.parametrize("mode", PE_MODES, ids=[m[0] for m in PE_MODES])
def test_match_fastq_paired_golden(gpu, pe_golden, tmp_path, gz, mode):
    """queryRoutinePaired over two mate files gives the reference's counters
    and tallies (MAXPDIST 550 fixtures)."""
    name, chunk, both = mode
    m1, m2 = golden_mates(pe_golden)
    p1, p2 = tmp_path / ("r1.fq.gz" if gz else "r1.fq"), tmp_path / ("r2.fq.gz" if gz else "r2.fq")
    write_fastq(p1, m1, gz)
    write_fastq(p2, m2, gz)
    gpu.tallies(reset=True)
    cnt, n = gpu.match_fastq_paired(str(p1), str(p2), gz, FAME_BOTH_STRANDS if both else 0,
                                    int(pe_golden["maxpdist"]), chunk=chunk, threads=3)
    ref = pe_golden[name + "_counters"]
    assert n == len(m1)
    assert pair_counters(cnt) == [int(x) for x in ref[:7]]
    assert np.array_equal(gpu.tallies(reset=True), pe_golden[name + "_meth"])


@pytest.mark.parametrize("npairs,chunk,both", [(3022, 1511, False),   # whole chunks: the last parse is empty
                                               (3000, 1000, True),
                                               (400, 1000, False)])
def test_match_fastq_paired_vs_chunk_loop(gpu, pe_golden, product_index, tmp_path, npairs, chunk, both):
    from fame_gb300 import PairedReadQueue
    m1, m2 = (m[:npairs] for m in golden_mates(pe_golden))
    p1, p2 = tmp_path / "r1.fq", tmp_path / "r2.fq"
    write_fastq(p1, m1, False)
    write_fastq(p2, m2, False)
    maxpdist = int(pe_golden["maxpdist"])
    gpu.tallies(reset=True)
    rq = PairedReadQueue(m1, m2, product_index, gpu, maxpdist=maxpdist, both_strands=both, chunk_size=chunk)
    tot = rq.query_routine_paired()
    exp_meth = gpu.tallies(reset=True)
    cnt, n = gpu.match_fastq_paired(str(p1), str(p2), False, FAME_BOTH_STRANDS if both else 0, maxpdist,
                                    chunk=chunk)
    assert n == npairs
    assert pair_counters(cnt)[:5] == [tot[k] for k in ("succ", "nonunique", "unsucc", "paired", "too_short")]
    assert (cnt.r1_fwd, cnt.r1_rev) == (rq.r1_fwd_matches, rq.r1_rev_matches)
    assert np.array_equal(gpu.tallies(reset=True), exp_meth)


def test_match_fastq_paired_errors(gpu, pe_golden, tmp_path):
    m1, m2 = golden_mates(pe_golden)
    p1, p2 = tmp_path / "r1.fq", tmp_path / "r2.fq"
    write_fastq(p1, m1[:500], False)
    write_fastq(p2, m2[:499], False)          # one mate missing
    with pytest.raises(FameError, match="different numbers"):
        gpu.match_fastq_paired(str(p1), str(p2), False, 0, 550, chunk=200)
    with pytest.raises(FameError):
        gpu.match_fastq_paired(str(p1), str(tmp_path / "missing.fq"), False, 0, 550)
    gpu.tallies(reset=True)
    write_fastq(p2, m2[:500], False)
    cnt, n = gpu.match_fastq_paired(str(p1), str(p2), False, 0, int(pe_golden["maxpdist"]))
    assert n == 500
    assert cnt.succ + cnt.unsucc + cnt.nonunique > 0
    gpu.tallies(reset=True)
