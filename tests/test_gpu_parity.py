"""Parity of the CUDA path (through the C ABI) with the reference and the oracle.

Bit-exact: per-read match (MATCH::match), invalid flag, every CpG tally and
the matchReads counters.  The golden values come from the compiled reference
(tests/golden/make_golden.py); the extra workloads are checked against the
oracle (oracle/fame_oracle.c), itself pinned to the reference.
"""
import numpy as np
import pytest

from fame_gb300 import (FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, FameError, GpuMatcher, HostIndex,
                        ReadQueue, synth)

pytestmark = pytest.mark.gpu

COMP = np.zeros(256, np.uint8)
for _a, _b in zip(b"ACGT", b"TGCA"):
    COMP[_a] = _b


@pytest.fixture(scope="module")
def gpu(product_index):
    g = GpuMatcher(product_index, 0)
    yield g
    g.close()


def run_mode(gpu, seq, offs, chunk, both):
    """queryRoutine's chunk loop (main.cpp:363-399) over fame_gpu_match_reads."""
    n = len(offs) - 1
    gpu.tallies(reset=True)
    mats = np.zeros(n, np.uint64)
    inval = np.zeros(n, np.uint8)
    tot = np.zeros(6, np.uint64)
    r1f = r1r = 0
    match_r1_fwd = True
    chunk = chunk or 300000
    for ci, c0 in enumerate(range(0, n, chunk)):
        c1 = min(n, c0 + chunk)
        stranded = ci == 0 and not both
        flags = (FAME_GET_STRANDED if stranded else 0) | (FAME_BOTH_STRANDS if both else 0) | \
            (FAME_MATCH_R1_FWD if match_r1_fwd else 0)
        o = offs[c0:c1 + 1].astype(np.uint64)
        m, iv, c = gpu.match_reads(seq[int(o[0]):int(o[-1])], o - o[0], flags)
        mats[c0:c1], inval[c0:c1] = m, iv
        tot[0] += c.succ
        tot[1] += c.nonunique
        tot[2] += c.unsucc
        r1f += c.r1_fwd
        r1r += c.r1_rev
        if stranded:
            match_r1_fwd = r1f > r1r
    tot[3], tot[4], tot[5] = r1f, r1r, int(match_r1_fwd)
    return dict(mat=mats, invalid=inval, meth=gpu.tallies(reset=True), counters=tot)


def assert_same(a, b, what=""):
    bad = np.nonzero((a["mat"] != b["mat"]) | (a["invalid"] != b["invalid"]))[0]
    assert len(bad) == 0, "%s: %d reads differ, first %s" % (what, len(bad), bad[:8])
    assert np.array_equal(a["meth"], b["meth"]), "%s: %d CpGs differ" % (what, int((a["meth"] != b["meth"]).any(1).sum()))
    assert np.array_equal(a["counters"], b["counters"]), "%s: %s vs %s" % (what, a["counters"], b["counters"])


@pytest.mark.parametrize("name,chunk,both", [("default", 0, False), ("chunk1000", 1000, False), ("both", 777, True)])
def test_golden_reference_parity(gpu, golden, name, chunk, both):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    r = run_mode(gpu, seq, offs, chunk, both)
    ref = {k: golden[name + "_" + k] for k in ("mat", "invalid", "meth", "counters")}
    assert_same(r, ref, name)


@pytest.mark.parametrize("mode", [1, 3], ids=["mid2048", "mid1024"])
@pytest.mark.parametrize("name,chunk,both", [("default", 0, False), ("chunk1000", 1000, False), ("both", 777, True)])
def test_golden_parity_middle_seeding_tier(gpu, golden, name, chunk, both, mode):
    """Every read seeded by the middle tiers (the genome-scale route: the
    shared-memory tier with either count-table size, then the global-memory
    ones) gives the reference's results too."""
    assert gpu.seed_tier() == 0
    gpu.seed_tier(mode)
    try:
        r = run_mode(gpu, golden["read_seq"].tobytes(), golden["read_offs"], chunk, both)
    finally:
        gpu.seed_tier(0)
    ref = {k: golden[name + "_" + k] for k in ("mat", "invalid", "meth", "counters")}
    assert_same(r, ref, name + " (middle tier, mode %d)" % mode)


def test_readqueue_mirror(golden, product_index, gpu):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    reads = [seq[int(offs[i]):int(offs[i + 1])] for i in range(len(offs) - 1)]
    gpu.tallies(reset=True)
    rq = ReadQueue(reads, product_index, gpu, chunk_size=1000)
    tot = rq.query_routine()
    c = golden["chunk1000_counters"]
    assert (tot["succ"], tot["nonunique"], tot["unsucc"]) == (c[0], c[1], c[2])
    assert int(rq.match_r1_fwd) == c[5]
    assert np.array_equal(rq.methylation_levels(), golden["chunk1000_meth"])
    gpu.tallies(reset=True)


@pytest.mark.parametrize("gz", [False, True], ids=["fastq", "fastq.gz"])
def test_readqueue_from_fastq_file(golden, product_index, gpu, tmp_path, gz):
    """The whole host flow from a FASTQ file (native chunk reader, GPU chunks,
    native report writer) gives the reference's counters and CpG report."""
    import gzip
    from fame_gb300 import write_cpg_report
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    lines = []
    for i in range(len(offs) - 1):
        r = seq[int(offs[i]):int(offs[i + 1])]
        lines += [b"@read%d" % i, r, b"+", b"I" * len(r)]
    path = tmp_path / ("reads.fq.gz" if gz else "reads.fq")
    with (gzip.open if gz else open)(path, "wb") as f:
        f.write(b"\n".join(lines) + b"\n")
    gpu.tallies(reset=True)
    rq = ReadQueue(str(path), product_index, gpu, is_gz=gz, chunk_size=1000)
    tot = rq.query_routine()
    c = golden["chunk1000_counters"]
    assert (tot["succ"], tot["nonunique"], tot["unsucc"]) == (c[0], c[1], c[2])
    report = tmp_path / "out"
    rq.print_methylation_levels(str(report))
    t = product_index.tables()
    names = product_index.chrom_names()
    m = golden["chunk1000_meth"]
    exp = "".join("%s\t%d\t%d\t%d\t%d\t%d\n" % (names[ch], p + 98, *m[i])
                  for i, (ch, p) in enumerate(zip(t["cpg_chrom"], t["cpg_pos"].astype(np.int64))))
    assert (tmp_path / "out_cpg.tsv").read_text() == exp
    gpu.tallies(reset=True)


def _oracle_run(oi, seq, offs, chunk=0, both=False):
    o = oi.match_se(seq, offs, chunk=chunk, both_strands=both)
    return dict(mat=o["mat"], invalid=o["invalid"], meth=o["meth"], counters=o["counters"])


def _workload(seed, n, readlen=100, lengths=None, err=0.02, indel=0.004, repeats=0.2, copies_div=(0.0, 0.08),
              chrom=(200_000, 120_000)):
    g = synth.make_genome(list(chrom), seed=seed, repeat_frac=repeats, n_families=12, fam_len=(300, 2000),
                          divergence=copies_div)
    rs = synth.make_reads(g, n, seed=seed + 1, read_len=readlen, sub_rate=err, indel_rate=indel,
                          length_sampler=lengths, repeat_read_frac=0.2)
    seqs = rs.seqs.copy()
    for i in range(0, n, 3):   # a third G->A converted
        s = seqs[i, : rs.lens[i]]
        seqs[i, : rs.lens[i]] = COMP[s[::-1]]
    reads = [seqs[i, : rs.lens[i]].tobytes() for i in range(n)]
    offs = np.zeros(n + 1, np.uint64)
    np.cumsum([len(r) for r in reads], out=offs[1:])
    return g, b"".join(reads), offs


@pytest.mark.parametrize("seed", [11, 12])
def test_oracle_parity_random(seed):
    from oracle.oracle import OracleIndex
    g, seq, offs = _workload(seed, 3000)
    hi = HostIndex.build(g.seqs, readlen=100)
    oi = OracleIndex.build(g.seqs, readlen=100)
    gm = GpuMatcher(hi, 0)
    try:
        for chunk, both in ((0, False), (500, False), (0, True)):
            assert_same(run_mode(gm, seq, offs, chunk, both), _oracle_run(oi, seq, offs, chunk, both),
                        "seed %d chunk %d both %d" % (seed, chunk, both))
    finally:
        gm.close()


def test_oracle_parity_read_lengths():
    """READLEN 150 index; reads of 80..255 bp exercise 2-, 3- and 4-word automata."""
    from oracle.oracle import OracleIndex

    def lens(rng, n):
        return rng.integers(125, 256, size=n)

    g, seq, offs = _workload(21, 2000, readlen=255, lengths=lens, chrom=(150_000, 90_000))
    hi = HostIndex.build(g.seqs, readlen=150)
    oi = OracleIndex.build(g.seqs, readlen=150)
    gm = GpuMatcher(hi, 0)
    try:
        assert_same(run_mode(gm, seq, offs, 0, True), _oracle_run(oi, seq, offs, 0, True), "lengths")
    finally:
        gm.close()


def test_oracle_parity_heavy_reads():
    """Near-identical repeat copies give reads hundreds to thousands of bucket
    entries, which pass through every seeding tier (the shared-memory middle
    tier, then the global-memory ones); the result must not change, whichever
    tier a read starts in and whatever the middle tier's table size."""
    from oracle.oracle import OracleIndex
    g, seq, offs = _workload(31, 1500, repeats=0.5, copies_div=(0.0, 0.005), chrom=(250_000,))
    hi = HostIndex.build(g.seqs, readlen=100)
    oi = OracleIndex.build(g.seqs, readlen=100)
    ref = _oracle_run(oi, seq, offs, 0, False)
    gm = GpuMatcher(hi, 0)
    try:
        for mode in range(4):
            gm.seed_tier(mode)
            assert_same(run_mode(gm, seq, offs, 0, False), ref, "heavy, seed mode %d" % mode)
    finally:
        gm.close()


def test_edge_cases(gpu):
    # empty chunk
    m, iv, c = gpu.match_reads(b"", np.zeros(1, np.uint64), FAME_GET_STRANDED)
    assert len(m) == 0 and c.succ == 0
    # all invalid: too short and N
    reads = [b"ACGT" * 10, b"N" * 120, b"ACGTN" * 30]
    offs = np.zeros(4, np.uint64)
    np.cumsum([len(r) for r in reads], out=offs[1:])
    m, iv, c = gpu.match_reads(b"".join(reads), offs, FAME_BOTH_STRANDS)
    assert list(iv) == [1, 1, 1] and list(m) == [0, 0, 0] and c.invalid_len == 1 and c.invalid_n == 2
    # reads beyond FAME_MAX_READ_LEN are refused with an error, not truncated
    reads = [b"ACGT" * 70]
    offs = np.array([0, 280], np.uint64)
    with pytest.raises(FameError) as e:
        gpu.match_reads(reads[0], offs, FAME_BOTH_STRANDS)
    assert e.value.code == -5
    gpu.tallies(reset=True)


def test_n_bases_at_word_edges(gpu, golden, oracle_index):
    """One N at the first, second, 8-byte-word-edge, middle and last bases of
    reads laid back to back at every byte alignment (the N check reads whole
    aligned words), mixed with clean reads; and the same chunk through the
    device entry point from a base address that is not word aligned."""
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"].astype(np.int64)
    reads = []
    for i in range(600):
        r = bytearray(seq[offs[i]:offs[i + 1]])
        L = len(r)
        pos = [0, 1, 7, 8, L // 2, L - 9, L - 8, L - 2, L - 1, -1][i % 10]
        if pos >= 0:
            r[pos] = ord("N")
        reads.append(bytes(r))
    o = np.zeros(len(reads) + 1, np.uint64)
    np.cumsum([len(r) for r in reads], out=o[1:])
    cat = b"".join(reads)
    got = run_mode(gpu, cat, o, 0, True)
    assert_same(got, _oracle_run(oracle_index, cat, o, 0, True), "N positions")
    with_n = np.array([b"N" in r for r in reads])
    assert got["invalid"][with_n].all() and with_n.sum() >= 540
    # device entry point, reads starting 3 bytes into an allocation
    n = len(reads)
    d_buf = gpu.alloc(len(cat) + 16)
    d_offs = gpu.alloc(8 * (n + 1))
    d_mat = gpu.alloc(8 * n)
    d_inv = gpu.alloc(n)
    try:
        gpu.memcpy(d_buf + 3, np.frombuffer(cat, np.uint8).ctypes.data, len(cat), 1)
        gpu.memcpy(d_offs, o.ctypes.data, 8 * (n + 1), 1)
        gpu.tallies(reset=True)
        gpu.match_reads_dev(d_buf + 3, d_offs, n, FAME_BOTH_STRANDS, d_mat, d_inv)
        mats = np.zeros(n, np.uint64)
        inv = np.zeros(n, np.uint8)
        gpu.memcpy(mats.ctypes.data, d_mat, 8 * n, 2)
        gpu.memcpy(inv.ctypes.data, d_inv, n, 2)
        meth = gpu.tallies(reset=True)
    finally:
        for p_ in (d_buf, d_offs, d_mat, d_inv):
            gpu.free(p_)
    assert np.array_equal(mats, got["mat"]) and np.array_equal(inv, got["invalid"])
    assert np.array_equal(meth, got["meth"])


def test_determinism_and_order(gpu, golden):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    a = run_mode(gpu, seq, offs, 0, True)
    b = run_mode(gpu, seq, offs, 0, True)
    assert_same(a, b, "repeat")
    n = len(offs) - 1
    perm = np.random.default_rng(0).permutation(n)
    reads = [seq[int(offs[i]):int(offs[i + 1])] for i in perm]
    po = np.zeros(n + 1, np.uint64)
    np.cumsum([len(r) for r in reads], out=po[1:])
    c = run_mode(gpu, b"".join(reads), po, 0, True)
    assert np.array_equal(c["mat"], a["mat"][perm]) and np.array_equal(c["invalid"], a["invalid"][perm])
    assert np.array_equal(c["meth"], a["meth"]) and np.array_equal(c["counters"], a["counters"])


def test_device_resident_entry_point(gpu, golden):
    seq = golden["read_seq"]
    offs = golden["read_offs"].astype(np.uint64)
    n = len(offs) - 1
    d_seq = gpu.alloc(len(seq))
    d_offs = gpu.alloc(8 * (n + 1))
    d_mat = gpu.alloc(8 * n)
    d_inv = gpu.alloc(n)
    try:
        gpu.memcpy(d_seq, seq.ctypes.data, len(seq), 1)
        gpu.memcpy(d_offs, offs.ctypes.data, 8 * (n + 1), 1)
        gpu.tallies(reset=True)
        cnt = gpu.match_reads_dev(d_seq, d_offs, n, FAME_BOTH_STRANDS, d_mat, d_inv)
        mats = np.zeros(n, np.uint64)
        inv = np.zeros(n, np.uint8)
        gpu.memcpy(mats.ctypes.data, d_mat, 8 * n, 2)
        gpu.memcpy(inv.ctypes.data, d_inv, n, 2)
        meth = gpu.tallies(reset=True)
    finally:
        for p in (d_seq, d_offs, d_mat, d_inv):
            gpu.free(p)
    ref = run_mode(gpu, seq.tobytes(), offs, 0, True)
    assert np.array_equal(mats, ref["mat"]) and np.array_equal(inv, ref["invalid"])
    assert np.array_equal(meth, ref["meth"]) and cnt.succ == ref["counters"][0]


def test_single_cell_batches(golden, product_index, gpu, oracle_index, tmp_path):
    """Two cells through SingleCellQueue: each cell's printed rows equal an
    independent run of the reference path on that cell's reads (votes restart
    per cell), and the bulk counters are left at zero."""
    from fame_gb300 import SingleCellQueue
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    reads = [seq[int(offs[i]):int(offs[i + 1])] for i in range(len(offs) - 1)]
    cells = [("cellA", reads[:2500]), ("cellB", reads[2500:])]
    gpu.tallies(reset=True)
    out = tmp_path / "sc.tsv"
    sc = SingleCellQueue(str(out), product_index, gpu, both_strands=False, chunk_size=1000)
    for cid, rr in cells:
        sc.match_sc_batch(rr, cid)
    sc.close()
    assert not gpu.tallies(reset=False).any()
    lines = out.read_text().split("\n")
    assert lines[0] == "" and lines[1].startswith("SC_ID\tCount_Type\t") and lines[2].startswith("SC_ID\tCount_Type\t")
    rows = {}
    for ln in lines[3:]:
        parts = ln.split("\t")
        rows[(parts[0], len([k for k in rows if k[0] == parts[0]]))] = np.array(parts[2:-1], dtype=np.int64)
    for cid, rr in cells:
        o = np.zeros(len(rr) + 1, np.uint64)
        np.cumsum([len(r) for r in rr], out=o[1:])
        ref = oracle_index.match_se(b"".join(rr), o, chunk=1000, both_strands=False)["meth"]
        for col in range(4):
            assert np.array_equal(rows[(cid, col)], ref[:, col].astype(np.int64)), (cid, col)


def test_device_map_orders_match_reference(gpu, kernels_golden):
    """The warp replay of tsl::hopscotch_map that orders a read's candidate
    windows, run on the device over the 400 adversarial key sequences whose
    iteration orders and final bucket counts the compiled reference's own map
    produced (tests/golden/make_golden.py): clustered keys, displacement
    chains, overflow lists and rehashes."""
    for c in kernels_golden["hopscotch"]:
        keys = np.asarray(c["keys"], np.uint32)
        _, first = np.unique(keys, return_index=True)
        distinct = keys[np.sort(first)]          # the map ignores repeated inserts
        order, fb = gpu.map_order_probe(distinct, int(c["bucket_count"]))
        assert np.array_equal(order, c["order"]), (len(keys), int(c["bucket_count"]))
        assert fb == int(c["final_buckets"])
