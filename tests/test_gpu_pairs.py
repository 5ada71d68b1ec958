"""Parity of the paired-end CUDA path (fame_gpu_match_pairs) with the reference
and the oracle: per-mate MATCH::match, isInvalid, every CpG tally and the
matchPairedReads counters, bit-exact.  The golden values come from the
compiled reference (tests/golden/make_golden_pe.py, MAXPDIST 550); the other
workloads are checked against the oracle, itself pinned to the reference."""
import numpy as np
import pytest

from fame_gb300 import (FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, HostIndex,
                        PairedReadQueue, synth)

pytestmark = pytest.mark.gpu

PE_MODES = (("default", 0, False), ("chunk700", 700, False), ("both", 900, True))
KEYS = ("mat1", "mat2", "inv1", "inv2", "meth", "counters")


@pytest.fixture(scope="module")
def gpu(product_index):
    g = GpuMatcher(product_index, 0)
    yield g
    g.close()


def run_pairs(gpu, s1, o1, s2, o2, chunk, both, maxpdist):
    """queryRoutinePaired's chunk loop (main.cpp:400-441) over fame_gpu_match_pairs."""
    n = len(o1) - 1
    gpu.tallies(reset=True)
    out = dict(mat1=np.zeros(n, np.uint64), mat2=np.zeros(n, np.uint64), inv1=np.zeros(n, np.uint8),
               inv2=np.zeros(n, np.uint8))
    tot = np.zeros(8, np.uint64)
    match_r1_fwd = True
    chunk = chunk or 300000
    heavy = 0
    for ci, c0 in enumerate(range(0, n, chunk)):
        c1 = min(n, c0 + chunk)
        stranded = ci == 0 and not both
        flags = (FAME_GET_STRANDED if stranded else 0) | (FAME_BOTH_STRANDS if both else 0) | \
            (FAME_MATCH_R1_FWD if match_r1_fwd else 0)
        a = o1[c0:c1 + 1].astype(np.uint64)
        b = o2[c0:c1 + 1].astype(np.uint64)
        m1, m2, i1, i2, c = gpu.match_pairs(s1[int(a[0]):int(a[-1])], a - a[0], s2[int(b[0]):int(b[-1])], b - b[0],
                                            flags, maxpdist)
        out["mat1"][c0:c1], out["mat2"][c0:c1], out["inv1"][c0:c1], out["inv2"][c0:c1] = m1, m2, i1, i2
        tot[:7] += np.array([c.succ, c.nonunique, c.unsucc, c.paired, c.too_short, c.r1_fwd, c.r1_rev], np.uint64)
        heavy += c.heavy_pairs
        if stranded:
            match_r1_fwd = tot[5] > tot[6]
    tot[7] = int(match_r1_fwd)
    out["meth"] = gpu.tallies(reset=True)
    out["counters"] = tot
    out["heavy"] = heavy
    return out


def assert_same(a, b, what):
    for k in ("mat1", "mat2", "inv1", "inv2"):
        bad = np.nonzero(a[k] != b[k])[0]
        assert len(bad) == 0, "%s: %s differs for %d pairs, first %s" % (what, k, len(bad), bad[:8])
    assert np.array_equal(a["meth"], b["meth"]), "%s: %d CpGs differ" % (what, int((a["meth"] != b["meth"]).any(1).sum()))
    assert np.array_equal(a["counters"], b["counters"]), (what, a["counters"], b["counters"])


def genome_of(seqs):
    return synth.Genome(names=["chr%d" % (i + 1) for i in range(len(seqs))], seqs=list(seqs),
                        meth=[np.zeros(len(x), bool) for x in seqs], repeat_copies=[])


def golden_pairs(g):
    return g["read_seq1"].tobytes(), g["read_offs1"], g["read_seq2"].tobytes(), g["read_offs2"]


@pytest.mark.parametrize("mode", PE_MODES, ids=[m[0] for m in PE_MODES])
def test_golden_modes(gpu, pe_golden, mode):
    name, chunk, both = mode
    s1, o1, s2, o2 = golden_pairs(pe_golden)
    got = run_pairs(gpu, s1, o1, s2, o2, chunk, both, int(pe_golden["maxpdist"]))
    assert_same(got, {k: pe_golden["%s_%s" % (name, k)] for k in KEYS}, name)


@pytest.mark.parametrize("mode", PE_MODES, ids=[m[0] for m in PE_MODES])
def test_golden_modes_middle_tier(gpu, pe_golden, mode):
    """Every pair seeded by the paired middle tier (the route genome-scale
    indexes take: global working memory with genome-scale caps, pairs from a
    work queue) gives the reference's results too."""
    name, chunk, both = mode
    s1, o1, s2, o2 = golden_pairs(pe_golden)
    assert gpu.seed_tier() == 0
    gpu.seed_tier(1)
    try:
        got = run_pairs(gpu, s1, o1, s2, o2, chunk, both, int(pe_golden["maxpdist"]))
    finally:
        gpu.seed_tier(0)
    assert_same(got, {k: pe_golden["%s_%s" % (name, k)] for k in KEYS}, name + " (middle tier)")


def test_paired_read_queue_mirror(gpu, pe_golden, product_index):
    """PairedReadQueue (the host mirror of the two-file ReadQueue) gives the
    reference's tallies and counters through the same C ABI."""
    s1, o1, s2, o2 = golden_pairs(pe_golden)
    mates = [[s[int(o[i]):int(o[i + 1])] for i in range(len(o) - 1)] for s, o in ((s1, o1), (s2, o2))]
    gpu.tallies(reset=True)
    rq = PairedReadQueue(mates[0], mates[1], product_index, gpu, maxpdist=int(pe_golden["maxpdist"]),
                         chunk_size=700)
    tot = rq.query_routine_paired()
    ref = pe_golden["chunk700_counters"]
    assert [tot["succ"], tot["nonunique"], tot["unsucc"], tot["paired"], tot["too_short"]] == [int(x) for x in ref[:5]]
    assert np.array_equal(gpu.tallies(reset=True), pe_golden["chunk700_meth"])


@pytest.mark.parametrize("seed,maxpdist", [(301, 550), (302, 400), (303, 2100)])
def test_oracle_random_pairs(gpu, oracle_index, golden_genome, seed, maxpdist):
    """Seeded pairs with 100, 150 and 230 bp mates (automaton widths 2, 3 and
    4; per-chunk k-mer arrays of 96, 160 and 224) at several MAXPDIST values
    (contextWLen 1 and 2) against the oracle."""
    g = genome_of(golden_genome)
    r1, r2 = synth.make_pairs(g, 1500, seed=seed, sub_rate=0.02, indel_rate=0.004,
                              inner=(20, maxpdist - 50))
    q1, q2 = synth.make_pairs(g, 300, seed=seed + 1000, read_len=150, inner=(20, 200))
    w1, w2 = synth.make_pairs(g, 80, seed=seed + 2000, read_len=230, inner=(20, 200))   # 4-word automaton
    s1, s2 = b"", b""
    o1 = o2 = np.zeros(1, np.uint64)
    for a, b in ((r1, r2), (q1, q2), (w1, w2)):
        sa, oa = a.concat()
        sb, ob = b.concat()
        s1, s2 = s1 + sa, s2 + sb
        o1 = np.concatenate([o1, oa[1:].astype(np.uint64) + o1[-1]])
        o2 = np.concatenate([o2, ob[1:].astype(np.uint64) + o2[-1]])
    for chunk, both in ((0, False), (600, False), (0, True)):
        got = run_pairs(gpu, s1, o1, s2, o2, chunk, both, maxpdist)
        ref = oracle_index.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=both, maxpdist=maxpdist)
        assert_same(got, ref, "seed %d maxpdist %d chunk %d both %d" % (seed, maxpdist, chunk, both))


def test_heavy_pairs_and_edge_cases():
    """A genome made of many copies of one segment: pairs there count hundreds
    of windows and run in the large-capacity launch; results equal the oracle.
    Also: an empty call, and every pair invalid."""
    from oracle.oracle import OracleIndex
    rng = np.random.default_rng(404)
    unit = synth.BASES[rng.integers(0, 4, 3000)]
    parts = []
    for i in range(150):
        parts.append(synth.BASES[rng.integers(0, 4, int(rng.integers(200, 2000)))])
        u = unit.copy()
        flip = rng.random(len(u)) < 0.01
        u[flip] = synth.BASES[rng.integers(0, 4, int(flip.sum()))]
        parts.append(u)
    chrom = np.concatenate(parts)
    cg = np.nonzero((chrom[:-1] == ord("C")) & (chrom[1:] == ord("G")))[0]
    chrom[cg[rng.random(len(cg)) < 0.5]] = ord("T")
    seqs = [chrom, synth.BASES[rng.integers(0, 4, 120_000)]]
    pidx = HostIndex.build(seqs, readlen=100)
    oidx = OracleIndex.build(seqs, readlen=100)
    g = genome_of(seqs)
    r1, r2 = synth.make_pairs(g, 600, seed=405, sub_rate=0.01, indel_rate=0.002)
    s1, o1 = r1.concat()
    s2, o2 = r2.concat()
    gpu = GpuMatcher(pidx, 0)
    try:
        heavy = 0
        for chunk, both in ((0, False), (0, True)):
            got = run_pairs(gpu, s1, o1, s2, o2, chunk, both, 550)
            ref = oidx.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=both, maxpdist=550)
            assert_same(got, ref, "repeat genome both %d" % both)
            heavy += got["heavy"]
        assert heavy > 0, "no pair exercised the large-capacity path"
        m1, m2, i1, i2, c = gpu.match_pairs(b"", np.zeros(1, np.uint64), b"", np.zeros(1, np.uint64), 0, 550)
        assert len(m1) == 0 and c.succ == 0
        bad = b"ACGTN" * 20
        o = np.array([0, 100, 200], np.uint64)
        m1, m2, i1, i2, c = gpu.match_pairs(bad + bad, o, b"ACGT" * 50, o, FAME_BOTH_STRANDS, 550)
        assert list(i1) == [1, 1] and list(i2) == [0, 0] and not m1.any() and not m2.any()
        assert c.too_short == 4 and c.succ == 0
    finally:
        gpu.close()
