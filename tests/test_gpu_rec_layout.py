"""Both layouts of the device's bucket records give the reference's results.

The dense layout (one 32-byte record per bucket, the genome-scale default)
and the hashed one (the non-empty buckets only, chosen by default for small
genomes) only change how a k-mer's bucket is found; every per-read match,
invalid flag, CpG tally and counter must stay the reference's, for single-end
and paired-end reads and through every seeding tier."""
import numpy as np
import pytest

from fame_gb300 import GpuMatcher, HostIndex
from test_gpu_pairs import KEYS as PE_KEYS, PE_MODES, assert_same as pe_same, golden_pairs, run_pairs
from test_gpu_parity import _oracle_run, _workload, assert_same, run_mode

pytestmark = pytest.mark.gpu

SE_MODES = (("default", 0, False), ("chunk1000", 1000, False), ("both", 777, True))
LAYOUTS = ((GpuMatcher.REC_DENSE, "dense"), (GpuMatcher.REC_HASHED, "hashed"))


@pytest.mark.parametrize("layout,lname", LAYOUTS, ids=[x[1] for x in LAYOUTS])
def test_golden_both_layouts(product_index, golden, pe_golden, layout, lname):
    g = GpuMatcher(product_index, 0, layout)
    try:
        got_layout, slots, nonempty = g.rec_layout()
        assert got_layout == layout
        assert 0 < nonempty <= product_index.view.n_kmer
        if layout == GpuMatcher.REC_HASHED:
            assert slots >= 2 * nonempty and slots & (slots - 1) == 0
        else:
            assert slots == 1 << 30
        seq, offs = golden["read_seq"].tobytes(), golden["read_offs"]
        for mode in (0, 1):   # the light tier first, then every read in the middle tiers
            g.seed_tier(mode)
            for name, chunk, both in SE_MODES:
                ref = {k: golden[name + "_" + k] for k in ("mat", "invalid", "meth", "counters")}
                assert_same(run_mode(g, seq, offs, chunk, both), ref, "%s %s tier %d" % (lname, name, mode))
            s1, o1, s2, o2 = golden_pairs(pe_golden)
            for name, chunk, both in PE_MODES:
                got = run_pairs(g, s1, o1, s2, o2, chunk, both, int(pe_golden["maxpdist"]))
                pe_same(got, {k: pe_golden["%s_%s" % (name, k)] for k in PE_KEYS}, "%s pairs %s" % (lname, name))
        g.seed_tier(0)
    finally:
        g.close()


def test_auto_layout_and_size(product_index):
    """A small genome's index takes the hashed layout by default, a small
    fraction of the dense one's 32 GiB of records."""
    auto = GpuMatcher(product_index, 0)
    try:
        layout, slots, nonempty = auto.rec_layout()
        assert layout == GpuMatcher.REC_HASHED
        hashed_bytes = auto.index_bytes()
    finally:
        auto.close()
    dense = GpuMatcher(product_index, 0, GpuMatcher.REC_DENSE)
    try:
        assert dense.rec_layout()[2] == nonempty
        assert dense.index_bytes() - hashed_bytes == 32 * ((1 << 30) - slots)
    finally:
        dense.close()


def test_heavy_reads_dense_layout():
    """Reads with hundreds to thousands of bucket entries (every seeding tier,
    including the global-memory ones that look buckets up by themselves) on
    the dense layout, against the oracle."""
    from oracle.oracle import OracleIndex
    g, seq, offs = _workload(31, 1500, repeats=0.5, copies_div=(0.0, 0.005), chrom=(250_000,))
    hi = HostIndex.build(g.seqs, readlen=100)
    ref = _oracle_run(OracleIndex.build(g.seqs, readlen=100), seq, offs, 0, False)
    gm = GpuMatcher(hi, 0, GpuMatcher.REC_DENSE)
    try:
        for mode in range(4):
            gm.seed_tier(mode)
            assert_same(run_mode(gm, seq, offs, 0, False), ref, "heavy, dense, seed mode %d" % mode)
    finally:
        gm.close()
