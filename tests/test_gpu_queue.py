"""The batched form (fame_queue_*, CUDA-graph chunk slots on their own
streams): bit-identical to the plain chunk calls, with chunks of several
slots in flight at once; per-job tally arrays give each job the same result
alone and interleaved with another job; a chunk whose candidates overflow
its slot is rerun by the plain path with the same results."""
import numpy as np
import pytest

from fame_gb300 import (FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, GpuQueue, HostIndex,
                        synth)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(product_index):
    g = GpuMatcher(product_index, 0)
    yield g
    g.close()


def chunks_of(offs, chunk):
    n = len(offs) - 1
    return [(c0, min(n, c0 + chunk)) for c0 in range(0, n, chunk)]


def run_queue(q, seq, offs, chunk, both, meth_dev=None):
    """queryRoutine's loop on the queue: chunk 0 (strand vote) first, then the
    rest with up to every slot in flight."""
    n = len(offs) - 1
    mats = np.zeros(n, np.uint64)
    inval = np.zeros(n, np.uint8)
    tot = np.zeros(3, np.uint64)
    cs = chunks_of(offs, chunk)

    def sub(a, b, flags):
        o = offs[a:b + 1].astype(np.uint64)
        return q.submit(seq[int(o[0]):int(o[-1])], o - o[0], flags, meth_dev)

    def col(slot, a, b):
        m, iv, c = q.collect(slot)
        mats[a:b], inval[a:b] = m, iv
        tot[:] += np.array([c.succ, c.nonunique, c.unsucc], np.uint64)
        return c

    r1f = r1r = 0
    start = 0
    match_r1_fwd = True
    if not both:
        a, b = cs[0]
        c = col(sub(a, b, FAME_GET_STRANDED), a, b)
        r1f, r1r = c.r1_fwd, c.r1_rev
        match_r1_fwd = r1f > r1r
        start = 1
    flags = (FAME_BOTH_STRANDS if both else 0) | (FAME_MATCH_R1_FWD if match_r1_fwd else 0)
    inflight = []
    for a, b in cs[start:]:
        if len(inflight) == q.nslots:
            s, a0, b0 = inflight.pop(0)
            col(s, a0, b0)
        inflight.append((sub(a, b, flags), a, b))
    for s, a0, b0 in inflight:
        col(s, a0, b0)
    return mats, inval, tot, (r1f, r1r, int(match_r1_fwd))


@pytest.mark.parametrize("mode", [("default", 6006, False), ("chunk1000", 1000, False), ("both", 777, True)],
                         ids=["default", "chunk1000", "both"])
def test_queue_matches_golden(gpu, golden, mode):
    name, chunk, both = mode
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    q = GpuQueue(gpu, 3, 6100, 6100 * 256)
    try:
        gpu.tallies(reset=True)
        mats, inval, tot, votes = run_queue(q, seq, offs, chunk, both)
    finally:
        q.close()
    assert np.array_equal(mats, golden["%s_mat" % name]) and np.array_equal(inval, golden["%s_invalid" % name])
    assert np.array_equal(gpu.tallies(reset=True), golden["%s_meth" % name])
    assert [int(x) for x in tot] == [int(x) for x in golden["%s_counters" % name][:3]]


def test_jobs_alone_and_mixed(gpu, golden):
    """Two jobs with their own tally arrays: interleaved on the queue, each
    ends with the tallies and matches it has when run alone."""
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    n = len(offs) - 1
    half = n // 2
    jobs = []
    for a, b in ((0, half), (half, n)):
        o = offs[a:b + 1].astype(np.uint64)
        jobs.append((seq[int(o[0]):int(o[-1])], o - o[0]))
    q = GpuQueue(gpu, 4, 800, 800 * 256)
    t_alone, t_mix = [], []
    try:
        alone = []
        for s, o in jobs:
            t = gpu.tally_alloc()
            alone.append(run_queue(q, s, o, 700, False, meth_dev=t))
            t_alone.append(t)
        # mixed: both jobs' chunks interleaved in the slots
        t_mix = [gpu.tally_alloc(), gpu.tally_alloc()]
        res = [dict(m=np.zeros(len(o) - 1, np.uint64), iv=np.zeros(len(o) - 1, np.uint8)) for _, o in jobs]
        state = []
        for j, (s, o) in enumerate(jobs):
            cs = chunks_of(o, 700)
            a, b = cs[0]
            oo = o[a:b + 1] - o[a]
            slot = q.submit(s[int(o[a]):int(o[b])], oo, FAME_GET_STRANDED, t_mix[j])
            state.append(dict(cs=cs, first=slot))
        for j, (s, o) in enumerate(jobs):
            a, b = state[j]["cs"][0]
            m, iv, c = q.collect(state[j]["first"])
            res[j]["m"][a:b], res[j]["iv"][a:b] = m, iv
            state[j]["flags"] = FAME_MATCH_R1_FWD if c.r1_fwd > c.r1_rev else 0
        work = [(j, a, b) for k in range(1, max(len(st["cs"]) for st in state))
                for j, st in enumerate(state) if k < len(st["cs"]) for a, b in [st["cs"][k]]]
        inflight = []
        for j, a, b in work:
            if len(inflight) == 4:
                slot, jj, a0, b0 = inflight.pop(0)
                m, iv, _ = q.collect(slot)
                res[jj]["m"][a0:b0], res[jj]["iv"][a0:b0] = m, iv
            s, o = jobs[j]
            slot = q.submit(s[int(o[a]):int(o[b])], o[a:b + 1] - o[a], state[j]["flags"], t_mix[j])
            inflight.append((slot, j, a, b))
        for slot, jj, a0, b0 in inflight:
            m, iv, _ = q.collect(slot)
            res[jj]["m"][a0:b0], res[jj]["iv"][a0:b0] = m, iv
        for j in range(2):
            assert np.array_equal(res[j]["m"], alone[j][0]) and np.array_equal(res[j]["iv"], alone[j][1])
            assert np.array_equal(gpu.tally_read(t_mix[j]), gpu.tally_read(t_alone[j]))
            assert gpu.tally_read(t_alone[j]).any()
    finally:
        q.close()
        for t in t_alone + t_mix:
            gpu.tally_free(t)


def test_candidate_overflow_rerun():
    """Reads from a genome of repeated segments have hundreds of candidate
    windows: the slot's candidate buffer overflows, the chunk is rerun by the
    plain path, and the results equal the plain call's."""
    rng = np.random.default_rng(505)
    unit = synth.BASES[rng.integers(0, 4, 3000)]
    parts = []
    for i in range(120):
        parts.append(synth.BASES[rng.integers(0, 4, int(rng.integers(100, 600)))])
        u = unit.copy()
        flip = rng.random(len(u)) < 0.005
        u[flip] = synth.BASES[rng.integers(0, 4, int(flip.sum()))]
        parts.append(u)
    seqs = [np.concatenate(parts)]
    idx = HostIndex.build(seqs, readlen=100)
    g = synth.Genome(names=["rep"], seqs=seqs, meth=[np.zeros(len(seqs[0]), bool)], repeat_copies=[])
    rs = synth.make_reads(g, 300, seed=506, sub_rate=0.01, indel_rate=0.001)
    s, o = rs.concat()
    gm = GpuMatcher(idx, 0)
    try:
        m_ref, iv_ref, c_ref = gm.match_reads(s, o, FAME_BOTH_STRANDS)
        t_ref = gm.tallies(reset=True)
        q = GpuQueue(gm, 2, 300, 300 * 256)
        slot = q.submit(s, o, FAME_BOTH_STRANDS)
        m, iv, c = q.collect(slot)
        q.close()
        assert c.windows_scanned > 2 * 300 * 4 + 4096, "the chunk did not overflow the slot"
        assert np.array_equal(m, m_ref) and np.array_equal(iv, iv_ref)
        assert (c.succ, c.nonunique, c.unsucc) == (c_ref.succ, c_ref.nonunique, c_ref.unsucc)
        assert np.array_equal(gm.tallies(reset=True), t_ref)
    finally:
        gm.close()


def test_bounded_wait_times_out_then_completes(gpu):
    """fame_queue_wait gives FAME_ERR_TIMEOUT while a chunk still runs (a zero
    timeout right after submitting 300k reads, whose copy alone takes longer),
    leaves the chunk running, and returns FAME_OK once it has finished; the
    collected results equal the plain call's."""
    g = synth.make_genome([400_000, 300_000], seed=61, repeat_frac=0.1, n_families=8, fam_len=(300, 1500))
    hi = HostIndex.build(g.seqs, readlen=100)
    gm = GpuMatcher(hi, 0)
    try:
        rs = synth.make_reads(g, 300_000, seed=62, sub_rate=0.01, indel_rate=0.001)
        seq, offs = rs.concat()
        q = GpuQueue(gm, 2, 300_000, len(seq))
        s = q.submit(seq, offs, FAME_MATCH_R1_FWD)
        assert q.wait(s, 0) is False            # FAME_ERR_TIMEOUT: still running
        assert q.wait(s, 60_000) is True        # finished within the minute
        m, iv, c = q.collect(s)
        q.close()
        m2, iv2, c2 = gm.match_reads(seq, offs, FAME_MATCH_R1_FWD)
        assert np.array_equal(m, m2) and np.array_equal(iv, iv2) and c.succ == c2.succ
    finally:
        gm.close()
