"""The native FASTQ chunk reader (fame_fastq_*) against parseChunk's rule —
four lines per record, the sequence is the second, nothing validated — on
plain and gzip files, uneven lengths, '@' and '+' inside quality lines, a
carriage return, no final newline, chunks that end inside a parse block, and
blocks larger than the reader's 64 MB buffer."""
import gzip

import numpy as np
import pytest

from fame_gb300._lib import FastqReader


def records(rng, n):
    out = []
    for i in range(n):
        L = int(rng.integers(0, 260))
        seq = rng.choice(np.frombuffer(b"ACGTN", np.uint8), L).tobytes()
        qual = rng.choice(np.frombuffer(b"@+IJ#", np.uint8), L).tobytes()
        out.append((b"@r%d extra" % i, seq, b"+" if i % 3 else b"+r%d" % i, qual))
    return out


def write(path, recs, gz=False, final_newline=True, crlf_at=None):
    lines = []
    for i, (h, s, p, q) in enumerate(recs):
        s2 = s + b"\r" if crlf_at == i else s
        lines += [h, s2, p, q]
    data = b"\n".join(lines) + (b"\n" if final_newline else b"")
    with (gzip.open if gz else open)(path, "wb") as f:
        f.write(data)


def read_all(path, gz, chunk, threads):
    r = FastqReader(str(path), is_gz=gz, n_threads=threads, max_reads=chunk, max_len=300)
    got = []
    while True:
        seq, offs = r.read()
        n = len(offs) - 1
        assert n <= chunk
        got += [bytes(seq[int(offs[i]):int(offs[i + 1])]) for i in range(n)]
        if n < chunk:
            break
    r.close()
    return got


@pytest.mark.parametrize("gz", [False, True])
@pytest.mark.parametrize("chunk,threads", [(1, 1), (7, 4), (1000, 3), (5000, 16)])
def test_reader_matches_parse_chunk(tmp_path, gz, chunk, threads):
    rng = np.random.default_rng(chunk + threads + gz)
    recs = records(rng, 3001)
    path = tmp_path / ("r.fq.gz" if gz else "r.fq")
    write(path, recs, gz=gz, final_newline=(chunk % 2 == 1), crlf_at=17)
    want = [s + (b"\r" if i == 17 else b"") for i, (_, s, _, _) in enumerate(recs)]
    assert read_all(path, gz, chunk, threads) == want


def test_reader_large_file(tmp_path):
    rng = np.random.default_rng(3)
    seq = rng.choice(np.frombuffer(b"ACGT", np.uint8), 150).tobytes()
    rec = b"@x\n" + seq + b"\n+\n" + b"I" * 150 + b"\n"
    n = (80 << 20) // len(rec) + 11                  # more than one 64 MB block
    path = tmp_path / "big.fq"
    with open(path, "wb") as f:
        f.write(rec * n)
    r = FastqReader(str(path), n_threads=8, max_reads=300000, max_len=160)
    total = 0
    while True:
        s, offs = r.read()
        k = len(offs) - 1
        assert np.all(np.diff(offs.astype(np.int64)) == 150)
        total += k
        if k < 300000:
            break
    r.close()
    assert total == n


@pytest.mark.parametrize("chunk,threads", [(1, 1), (999, 4)])
def test_reader_pipe(tmp_path, chunk, threads):
    """A named pipe cannot be mapped: the buffered path, same records."""
    import os
    import threading
    rng = np.random.default_rng(7 + chunk)
    recs = records(rng, 2500)
    data_path = tmp_path / "src.fq"
    write(data_path, recs, final_newline=False)
    fifo = tmp_path / "pipe.fq"
    os.mkfifo(fifo)

    def feed():
        with open(fifo, "wb") as f:
            f.write(data_path.read_bytes())

    th = threading.Thread(target=feed)
    th.start()
    got = read_all(fifo, False, chunk, threads)
    th.join()
    assert got == [s for _, s, _, _ in recs]


def test_reader_empty_and_tiny(tmp_path):
    empty = tmp_path / "e.fq"
    empty.write_bytes(b"")
    assert read_all(empty, False, 10, 4) == []
    one = tmp_path / "one.fq"
    one.write_bytes(b"@a\nACGT")          # a record cut after its sequence line
    assert read_all(one, False, 10, 4) == [b"ACGT"]
    blank = tmp_path / "blank.fq"
    blank.write_bytes(b"\n\n\n\n\n\n")     # empty lines are lines: two records of empty sequences
    assert read_all(blank, False, 10, 2) == [b"", b""]


@pytest.mark.parametrize("gz", [False, True])
def test_two_readers_at_once(tmp_path, gz):
    """Two readers used from two threads at the same time (the paired
    pipeline reads both mate files so) give each file's records."""
    import threading
    rng = np.random.default_rng(11)
    recs = [records(rng, 1500), records(rng, 1500)]
    paths = [tmp_path / ("m%d.fq%s" % (m, ".gz" if gz else "")) for m in (1, 2)]
    for p, r in zip(paths, recs):
        write(p, r, gz=gz)
    got = [None, None]

    def run(m):
        got[m] = read_all(paths[m], gz, 400, 3)

    th = [threading.Thread(target=run, args=(m,)) for m in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert got == [[s for _, s, _, _ in r] for r in recs]
