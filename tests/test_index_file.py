"""The --load_index file format (RefGenome::save / load, RefGenome.cpp:83-433).

The product's writer (fame_index_write) against the file the reference's own
RefGenome::save writes for the same genome, byte for byte apart from the
struct padding bytes (uninitialised in the reference), the _strands side
file exactly; and the product's reader (fame_index_read) on the reference's
file against the product's own build.  The genome carries tandem repeats, so
that k-mers pass KMERCUTOFF and the filtered-k-mer set (an unordered_set in
the reference, written in its iteration order) is not empty.

Needs the compiled reference (oracle/_ref, built by build() where the
reference sources are present); skipped elsewhere.  Each file holds an 8 GiB
offset table; both are deleted at the end.
"""
import os

import numpy as np
import pytest

from oracle import refbind

pytestmark = pytest.mark.skipif(not refbind.available(), reason="compiled reference (oracle/_ref) not built")

HTABSIZE = 1 << 30


def make_genome():
    rng = np.random.default_rng(2024)
    acgt = np.frombuffer(b"ACGT", np.uint8)

    def rnd(n):
        return rng.choice(acgt, n, p=[0.295, 0.205, 0.205, 0.295])

    def tandem(unit, copies):
        return np.tile(rnd(unit), copies)

    chr1 = np.concatenate([rnd(150_000), tandem(41, 6_000), rnd(100_000)])
    chr2 = np.concatenate([rnd(120_000), np.full(5_000, ord("N"), np.uint8), tandem(67, 3_500), rnd(60_000)])
    chr3 = np.concatenate([rnd(80_000), tandem(29, 7_000), rnd(40_000)])
    return [chr1.astype(np.uint8), chr2.astype(np.uint8), chr3.astype(np.uint8)], ["chr1", "chrB", "scaffold_3"]


def sections(buf):
    """Byte ranges of the padded struct arrays: (start, count, record size, padding offsets)."""
    o = 32                                    # u64 HTABSIZE, u32 READLEN, WINLEN, KMERLEN, u64 KMERCUTOFF, u32 SEEDBITS
    out = []
    for _ in range(2):                        # CpGs, start CpGs: {u8 chrom, 3 padding, u32 pos}
        n = int(buf[o:o + 8].view(np.uint64)[0])
        out.append((o + 8, n, 8, (1, 2, 3)))
        o += 8 + 8 * n
    nch = int(buf[o:o + 8].view(np.uint64)[0])
    o += 8
    for _ in range(nch):
        o += 8 + int(buf[o:o + 8].view(np.uint64)[0])
    tab = int(buf[o:o + 8].view(np.uint64)[0])
    assert tab == HTABSIZE + 1
    o += 8 + 8 * tab
    nk = int(buf[o:o + 8].view(np.uint64)[0])
    kstart = o + 8
    o += 8 + 8 * nk
    for _ in range(2):                        # metaCpGs, start metaCpGs: empty
        assert int(buf[o:o + 8].view(np.uint64)[0]) == 0
        o += 8
    nw = int(buf[o:o + 8].view(np.uint64)[0])
    out.append((o + 8, nw, 16, (5, 6, 7)))    # {u32 start, u8 chrom, 3 padding, u32 sind, u32 eind}
    o += 8 + 16 * nw
    nf = int(buf[o:o + 8].view(np.uint64)[0])
    return out, kstart, nk, nf


def assert_same_file(ours, theirs, skip):
    """Equal bytes except at the positions in skip."""
    a = np.memmap(ours, np.uint8, mode="r")
    b = np.memmap(theirs, np.uint8, mode="r")
    assert a.size == b.size
    pad = np.sort(skip)
    step = 256 << 20
    for s in range(0, a.size, step):
        x = np.array(a[s:s + step])
        y = np.array(b[s:s + step])
        p = pad[(pad >= s) & (pad < s + step)] - s
        x[p] = 0
        y[p] = 0
        if not np.array_equal(x, y):
            first = int(np.nonzero(x != y)[0][0]) + s
            raise AssertionError("files differ at byte %d" % first)


def test_index_file_matches_reference_save(tmp_path):
    from fame_gb300 import HostIndex
    seqs, names = make_genome()
    fasta = tmp_path / "genome.fa"
    with open(fasta, "wb") as f:
        for nm, s in zip(names, seqs):
            f.write(b">" + nm.encode() + b" description\n")
            for i in range(0, len(s), 70):
                f.write(s[i:i + 70].tobytes() + b"\n")
    ref_path, our_path = str(tmp_path / "ref.idx"), str(tmp_path / "ours.idx")
    try:
        L = refbind.RefLib()
        L.lib.fame_ref_build_save.argtypes = [refbind.C.c_char_p, refbind.C.c_int, refbind.C.c_char_p]
        assert L.lib.fame_ref_build_save(str(fasta).encode(), 0, ref_path.encode()) == 0
        hi = HostIndex.build(seqs, readlen=100, names=names)
        built = hi.tables()
        assert len(built["filtered"]) > 10, "the tandem repeats should pass KMERCUTOFF"
        hi.write(our_path)
        masked, kstart, nk, nf = sections(np.memmap(our_path, np.uint8, mode="r"))
        assert nk == len(built["kmer_meta"]) and nf == len(built["filtered"])
        # T masks the reference reads past a chromosome's end (reverse-strand
        # k-mers of a truncated last window; the bytes there are whatever
        # memory follows the sequence): left out of the comparison
        lens = np.array([len(x) for x in seqs], np.int64)
        w_end = built["win_start"].astype(np.int64) + 2048
        truncated = np.nonzero(w_end > lens[built["win_chrom"]])[0]
        loose = np.nonzero(np.isin(built["kmer_meta"] & 0x7fffffff, truncated))[0]
        assert len(loose) < nk // 100
        skip = [start + rec * np.arange(n, dtype=np.int64) + k for start, n, rec, offs in masked for k in offs]
        skip += [kstart + 8 * loose.astype(np.int64) + k for k in (4, 5, 6, 7)]
        assert_same_file(our_path, ref_path, np.concatenate(skip))
        with open(our_path + "_strands", "rb") as f1, open(ref_path + "_strands", "rb") as f2:
            assert f1.read() == f2.read()
        hi.close()
        # the reader on the reference's file gives the product's own build
        back = HostIndex.read(ref_path)
        got = back.tables()
        keep = np.ones(nk, bool)
        keep[loose] = False
        for k, v in built.items():
            if k == "kmer_tmask":
                assert np.array_equal(got[k][keep], v[keep]), k
            else:
                assert np.array_equal(got[k], v), k
        assert back.chrom_names() == names
        assert [bytes(s) for s in back.chrom_seqs()] == [s.tobytes() for s in seqs]
        back.close()
    finally:
        for p in (ref_path, our_path):
            for q in (p, p + "_strands"):
                if os.path.exists(q):
                    os.remove(q)
