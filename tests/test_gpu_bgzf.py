"""BGZF input inflated on the GPU (fame_fastq_open_dev; one warp per gzip
member, every member's size and CRC-32 checked): the records equal the plain
file's for stored, fast and best compression, members from a few hundred
bytes to 64 KiB and chunks that end inside a member; a flipped byte or a
truncated file fails the read; plain gzip still goes through zlib; and the
whole-file pipeline on a BGZF file gives the plain file's tallies and
counters."""
import numpy as np
import pytest

from bgzf_writer import bgzf
from fame_gb300 import FameError, FAME_GET_STRANDED, GpuMatcher
from fame_gb300._lib import FastqReader
from test_fastq import records

pytestmark = pytest.mark.gpu


def fastq_bytes(recs):
    return b"\n".join(x for r in recs for x in r) + b"\n"


def read_gpu(path, chunk, threads=3, expect_gpu=True):
    r = FastqReader(str(path), is_gz=True, n_threads=threads, max_reads=chunk, max_len=300, device=0)
    assert r.gpu_inflate == expect_gpu
    got = []
    try:
        while True:
            seq, offs = r.read()
            n = len(offs) - 1
            got += [bytes(seq[int(offs[i]):int(offs[i + 1])]) for i in range(n)]
            if n < chunk:
                break
    finally:
        r.close()
    return got


@pytest.mark.parametrize("level,block", [(0, 65280), (1, 400), (6, 65280), (9, 7000)])
@pytest.mark.parametrize("chunk", [13, 1000, 100000])
def test_records_equal_plain(tmp_path, level, block, chunk):
    rng = np.random.default_rng(level * 100 + chunk)
    recs = records(rng, 6000)
    p = tmp_path / "r.fq.gz"
    p.write_bytes(bgzf(fastq_bytes(recs), level, block))
    assert read_gpu(p, chunk) == [s for _, s, _, _ in recs]


def test_large_file_many_members(tmp_path):
    """Far more than one refill of compressed input (64 MiB pieces)."""
    rng = np.random.default_rng(5)
    alpha = np.frombuffer(b"ACGT", np.uint8)
    seqs = [rng.choice(alpha, 150).tobytes() for _ in range(20000)]
    data = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, s, b"I" * 150) for i, s in enumerate(seqs))
    big = data * 40   # about 280 MB of text
    p = tmp_path / "big.fq.gz"
    p.write_bytes(bgzf(big, 1))
    got = read_gpu(p, 300000)
    assert len(got) == 800000 and got[:20000] == seqs and got[-20000:] == seqs


def test_corrupt_and_truncated(tmp_path):
    rng = np.random.default_rng(6)
    recs = records(rng, 4000)
    b = bytearray(bgzf(fastq_bytes(recs), 6, 20000))
    bad = bytearray(b)
    bad[len(b) // 2] ^= 0x5A   # inside a member's compressed data (or its header)
    p = tmp_path / "bad.fq.gz"
    p.write_bytes(bytes(bad))
    with pytest.raises(FameError):
        read_gpu(p, 100000)
    t = tmp_path / "trunc.fq.gz"
    t.write_bytes(bytes(b[: len(b) - 5000]))
    with pytest.raises(FameError):
        read_gpu(t, 100000)


def test_plain_gzip_uses_zlib(tmp_path):
    import gzip
    rng = np.random.default_rng(7)
    recs = records(rng, 3000)
    p = tmp_path / "plain.fq.gz"
    p.write_bytes(gzip.compress(fastq_bytes(recs)))
    assert read_gpu(p, 1000, expect_gpu=False) == [s for _, s, _, _ in recs]


def test_pipeline_on_bgzf(tmp_path, golden, product_index):
    """fame_match_fastq over a BGZF copy of the golden reads equals the plain file."""
    seq, offs = golden["read_seq"].tobytes(), golden["read_offs"]
    n = len(offs) - 1
    text = b"".join(b"@r%d\n%s\n+\n%s\n" % (i, seq[int(offs[i]):int(offs[i + 1])], b"I" * int(offs[i + 1] - offs[i]))
                    for i in range(n))
    plain = tmp_path / "g.fq"
    plain.write_bytes(text)
    bz = tmp_path / "g.fq.gz"
    bz.write_bytes(bgzf(text, 6, 5000))
    gm = GpuMatcher(product_index, 0)
    try:
        res = []
        for path, gz in ((plain, False), (bz, True)):
            gm.tallies(reset=True)
            c, nr = gm.match_fastq(str(path), gz, FAME_GET_STRANDED, chunk=700)
            res.append((c.succ, c.nonunique, c.unsucc, c.r1_fwd, c.r1_rev, nr, gm.tallies(reset=True)))
        assert res[0][:6] == res[1][:6]
        assert np.array_equal(res[0][6], res[1][6])
    finally:
        gm.close()
