"""Parity at the scale of the smallest benchmark workload: the 20 Mbp genome
(4 x 5 Mbp, seed 1) with 100k single-end reads of 100 bp, and 20k read pairs
on the same genome, through the C ABI against the compiled reference.

The reference side is FAME's own code (oracle/_ref: its readReference +
RefGenome constructor build the index from a FASTA of the genome, and its
matchReads / matchPairedReads chunk loops run the reads); the GPU side builds
its index with fame_index_build.  So this pins the index build, the upload
and every kernel end to end, bit for bit: per-read MATCH::match and
isInvalid, every uint16 CpG tally and the counters, in the three run modes of
queryRoutine (strand vote on the first chunk, several chunks, --unord_reads).
Where the reference library is not built, the C restatement (oracle/) is the
checker instead.
"""
import numpy as np
import pytest

from fame_gb300 import (FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, HostIndex, synth)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def workload():
    spec = synth.WORKLOADS["se100_20mbp"]
    g = synth.make_genome(**spec["genome"])
    rs = synth.make_reads(g, **spec["reads"])
    seq, offs = rs.concat()
    p1, p2 = synth.make_pairs(g, 20_000, seed=3, sub_rate=0.01, indel_rate=0.001)
    return g, seq, offs, p1.concat(), p2.concat()


@pytest.fixture(scope="module")
def checker(workload, tmp_path_factory):
    """(kind, index handle) of the reference built from the genome's FASTA, else the oracle."""
    g = workload[0]
    try:
        from oracle import refbind
        if refbind.available():
            L = refbind.RefLib()
            if L.readlen == 100:
                fa = str(tmp_path_factory.mktemp("cfg0") / "genome.fa")
                g.write_fasta(fa)
                ri = L.build(fa)
                yield "reference", ri, L.maxpdist()
                ri.close()
                return
    except OSError:
        pass
    from oracle.oracle import OracleIndex
    yield "oracle", OracleIndex.build(g.seqs, readlen=100), 550


@pytest.fixture(scope="module")
def gpu(workload):
    hi = HostIndex.build(workload[0].seqs, readlen=100, threads=0)
    gm = GpuMatcher(hi, 0)
    yield gm
    gm.close()


def gpu_query_routine(gm, seq, offs, chunk, both):
    """queryRoutine's chunk loop (main.cpp:363-399) over fame_gpu_match_reads."""
    n = len(offs) - 1
    gm.tallies(reset=True)
    mats = np.zeros(n, np.uint64)
    inval = np.zeros(n, np.uint8)
    tot = np.zeros(6, np.uint64)
    r1f = r1r = 0
    fwd = True
    for ci, c0 in enumerate(range(0, n, chunk)):
        c1 = min(n, c0 + chunk)
        stranded = ci == 0 and not both
        flags = (FAME_GET_STRANDED if stranded else 0) | (FAME_BOTH_STRANDS if both else 0) | \
            (FAME_MATCH_R1_FWD if fwd else 0)
        o = offs[c0:c1 + 1].astype(np.uint64)
        m, iv, c = gm.match_reads(seq[int(o[0]):int(o[-1])], o - o[0], flags)
        mats[c0:c1], inval[c0:c1] = m, iv
        tot[0] += c.succ
        tot[1] += c.nonunique
        tot[2] += c.unsucc
        r1f += c.r1_fwd
        r1r += c.r1_rev
        if stranded:
            fwd = r1f > r1r
    tot[3], tot[4], tot[5] = r1f, r1r, int(fwd)
    return dict(mat=mats, invalid=inval, meth=gm.tallies(reset=True), counters=tot)


@pytest.mark.parametrize("mode,chunk,both", [("strand_vote", 300_000, False), ("chunks_of_30k", 30_000, False),
                                             ("unord_reads", 45_000, True)])
def test_single_end_100k_reads_20mbp(workload, checker, gpu, mode, chunk, both):
    _, seq, offs, _, _ = workload
    kind, ref_ix, _ = checker
    ref = ref_ix.match_se(seq, offs, chunk=chunk, both_strands=both)
    got = gpu_query_routine(gpu, seq, offs, chunk, both)
    bad = np.flatnonzero((got["mat"] != ref["mat"]) | (got["invalid"] != ref["invalid"]))
    assert len(bad) == 0, "%s vs %s: %d of %d reads differ, first %s" % (mode, kind, len(bad), len(offs) - 1, bad[:8])
    nbad = int((got["meth"] != ref["meth"]).any(1).sum())
    assert nbad == 0, "%s vs %s: %d CpGs differ" % (mode, kind, nbad)
    assert np.array_equal(got["counters"], np.asarray(ref["counters"][:6], np.uint64)), \
        "%s vs %s: counters %s vs %s" % (mode, kind, got["counters"], ref["counters"])
    # 0.5x coverage: about 40 % of the CpGs see a read
    assert got["counters"][0] > 99_000 and int((got["meth"] > 0).any(1).sum()) > 0.3 * len(got["meth"])


def test_paired_end_20k_pairs_20mbp(workload, checker, gpu):
    """queryRoutinePaired's chunk loop (main.cpp:400-441) in chunks of 7,000
    pairs, strand vote on the first, at the reference library's MAXPDIST."""
    _, _, _, (s1, o1), (s2, o2) = workload
    kind, ref_ix, maxpdist = checker
    chunk = 7_000
    if kind == "reference":
        ref = ref_ix.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=False)
    else:
        ref = ref_ix.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=False, maxpdist=maxpdist)
    n = len(o1) - 1
    gpu.tallies(reset=True)
    got = dict(mat1=np.zeros(n, np.uint64), mat2=np.zeros(n, np.uint64), inv1=np.zeros(n, np.uint8),
               inv2=np.zeros(n, np.uint8))
    tot = np.zeros(8, np.uint64)
    fwd = True
    for ci, c0 in enumerate(range(0, n, chunk)):
        c1 = min(n, c0 + chunk)
        flags = FAME_GET_STRANDED if ci == 0 else (FAME_MATCH_R1_FWD if fwd else 0)
        a1 = o1[c0:c1 + 1].astype(np.uint64)
        a2 = o2[c0:c1 + 1].astype(np.uint64)
        m1, m2, i1, i2, c = gpu.match_pairs(s1[int(a1[0]):int(a1[-1])], a1 - a1[0], s2[int(a2[0]):int(a2[-1])],
                                            a2 - a2[0], flags, maxpdist)
        got["mat1"][c0:c1], got["mat2"][c0:c1], got["inv1"][c0:c1], got["inv2"][c0:c1] = m1, m2, i1, i2
        tot[:7] += np.array([c.succ, c.nonunique, c.unsucc, c.paired, c.too_short, c.r1_fwd, c.r1_rev], np.uint64)
        if ci == 0:
            fwd = tot[5] > tot[6]
    tot[7] = int(fwd)
    meth = gpu.tallies(reset=True)
    for k in ("mat1", "mat2", "inv1", "inv2"):
        bad = np.flatnonzero(got[k] != ref[k])
        assert len(bad) == 0, "%s vs %s: %d pairs differ, first %s" % (k, kind, len(bad), bad[:8])
    assert np.array_equal(meth, ref["meth"]), "%d CpGs differ" % int((meth != ref["meth"]).any(1).sum())
    assert np.array_equal(tot, np.asarray(ref["counters"], np.uint64)), (tot, ref["counters"])
    assert tot[3] > 15_000   # pairs with both mates in CpG windows
