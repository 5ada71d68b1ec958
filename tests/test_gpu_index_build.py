"""The index built on the GPU (fame_index_build_gpu) against the host build
(fame_index_build, itself pinned to the reference's tables and files): every
table identical -- bucket offsets, k-mer entries and T masks, strandTable,
windows, CpGs, the filtered k-mers and the order the reference's set
received them.  The genomes cover N runs (the forward buffer's mirrored N
stores), chromosomes shorter than a read, READLEN 100 and 150, repeat
families (buckets for the shared-memory pass), tandem repeats past
KMERCUTOFF (the filter and the global-scratch pass), and the noloss build."""
import hashlib

import numpy as np
import pytest

from fame_gb300 import HostIndex, synth

pytestmark = pytest.mark.gpu

HTABSIZE = 1 << 30


def tab32(hi):
    return hi._arr(hi.view.tab_index32, HTABSIZE + 1, np.uint32)


def assert_same_index(a, b, what):
    ta, tb = a.tables(sparse=False), b.tables(sparse=False)
    for k in ta:
        assert np.array_equal(ta[k], tb[k]), "%s: %s differs" % (what, k)
    assert np.array_equal(tab32(a), tab32(b)), "%s: bucket offsets differ" % what
    assert np.array_equal(a.filtered_order(), b.filtered_order()), "%s: filtered k-mer order differs" % what
    assert a.chrom_names() == b.chrom_names()
    assert all(np.array_equal(x, y) for x, y in zip(a.chrom_seqs(), b.chrom_seqs()))
    return ta


def build_both(seqs, readlen, names=None, noloss=False):
    host = HostIndex.build(seqs, readlen=readlen, names=names, noloss=noloss)
    dev = HostIndex.build_gpu(seqs, readlen=readlen, names=names, noloss=noloss, device=0)
    return host, dev


def test_golden_genome(golden, golden_genome, product_index):
    dev = HostIndex.build_gpu(golden_genome, readlen=100)
    try:
        assert_same_index(dev, product_index, "golden genome")
        dig = golden["digests"].item()
        t = dev.tables()
        for k in ("cpg_pos", "bucket_key", "bucket_start", "kmer_meta", "strand", "win_sind", "win_eind"):
            assert hashlib.sha256(np.ascontiguousarray(t[k]).tobytes()).hexdigest() == dig[k], k
    finally:
        dev.close()


@pytest.mark.parametrize("readlen", [100, 150])
def test_n_runs_and_short_chromosomes(readlen):
    rng = np.random.default_rng(77 + readlen)

    def chrom(n, nfrac):
        s = synth.BASES[rng.integers(0, 4, n)].copy()
        for _ in range(int(n * nfrac / 20)):
            p = int(rng.integers(0, n))
            s[p:p + int(rng.integers(1, 60))] = ord("N")
        return s

    seqs = [chrom(90_000, 0.02), chrom(150, 0.0), chrom(50_000, 0.0), chrom(77_777, 0.05), chrom(2047, 0.01)]
    seqs[2][:3000] = ord("N")
    seqs[2][-2500:] = ord("N")
    host, dev = build_both(seqs, readlen)
    try:
        t = assert_same_index(dev, host, "N runs, READLEN %d" % readlen)
        assert len(t["kmer_meta"]) > 10_000
    finally:
        host.close()
        dev.close()


def test_repeat_families():
    g = synth.make_genome([300_000, 200_000], seed=88, repeat_frac=0.4, n_families=6, fam_len=(300, 2000),
                          divergence=(0.0, 0.01))
    host, dev = build_both(g.seqs, 100)
    try:
        t = assert_same_index(dev, host, "repeat families")
        ln = np.diff(tab32(host).astype(np.int64))
        assert (ln > 16).sum() > 0, "no bucket for the shared-memory pass"
    finally:
        host.close()
        dev.close()


@pytest.mark.parametrize("noloss", [False, True], ids=["filtered", "noloss"])
def test_tandem_repeats_past_kmercutoff(noloss):
    from test_index_file import make_genome
    seqs, names = make_genome()
    host, dev = build_both(seqs, 100, names=names, noloss=noloss)
    try:
        t = assert_same_index(dev, host, "tandem repeats, noloss %d" % noloss)
        if noloss:   # raw buckets of thousands of entries: the global-scratch pass without the k-mer filter
            assert len(t["filtered"]) == 0
        else:
            assert len(t["filtered"]) > 10, "the tandem repeats should pass KMERCUTOFF"
    finally:
        host.close()
        dev.close()
