"""GPU test of fame_gpu_call_cpgs_noalloc, the entry point that allocates no
device memory (for callers that cannot allocate while they run, for example
a serving loop that must not stall its other streams on cudaFree's implicit
device synchronisation).

It is called through the C ABI on caller-owned device buffers and must give
the same CpG counters as the regular entry point (fame_gpu_match_reads +
fame_gpu_tallies) on the same reads, exactly, on two calls in a row (the
static scratch array keeps the previous call's contents).  This file sorts
last so that a run stopping at the first failure has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

from fame_gb300 import FAME_MATCH_R1_FWD, GpuMatcher, HostIndex, lib, synth

pytestmark = pytest.mark.gpu


def _entry_point():
    f = lib().fame_gpu_call_cpgs_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_cpg_calls_match_regular_entry_point():
    g = synth.make_genome([150_000, 80_000], seed=41, repeat_frac=0.1, n_families=8, fam_len=(300, 1500))
    rs = synth.make_reads(g, 4000, seed=42, sub_rate=0.02, indel_rate=0.004)
    seq, offs = rs.concat()
    n = len(offs) - 1
    hi = HostIndex.build(g.seqs, readlen=100)
    gm = GpuMatcher(hi, 0)
    bufs = []
    try:
        # regular entry point: forward orientation (the decided strand), tallies
        gm.tallies(reset=True)
        mats, inval, cnt = gm.match_reads(seq, offs, FAME_MATCH_R1_FWD)
        expect = gm.tallies(reset=True)
        assert cnt.succ > 3000 and cnt.dp_reads > 500  # exact hits and banded-DP hits both present
        ncpg = gm.n_cpg
        # the caller's device buffers (allocated here by the test, not by the entry point)
        raw = np.frombuffer(seq, np.uint8)
        d_seq, d_offs, d_mats, d_inv, d_meth = (gm.alloc(b) for b in (len(raw), 8 * (n + 1), 8 * n, n, 16 * ncpg))
        bufs = [d_seq, d_offs, d_mats, d_inv, d_meth]
        gm.memcpy(d_seq, raw.ctypes.data, len(raw), 1)
        gm.memcpy(d_offs, offs.ctypes.data, 8 * (n + 1), 1)
        gm.memcpy(d_mats, mats.ctypes.data, 8 * n, 1)
        gm.memcpy(d_inv, inval.ctypes.data, n, 1)
        f = _entry_point()
        for call in range(2):
            assert f(gm.h, d_seq, d_offs, d_mats, d_inv, n, 0, d_meth) == 0
            got = np.zeros(4 * ncpg, np.uint32)
            gm.memcpy(got.ctypes.data, d_meth, 16 * ncpg, 2)
            assert np.array_equal((got & 0xFFFF).astype(np.uint16).reshape(-1, 4), expect), "call %d" % call
        # reverse orientation (orient 1): the reverse complements of the same
        # reads, matched with matchR1Fwd false (each read reverse-complemented
        # back before matching), so the same hits, DP ones included
        rc = np.concatenate([synth._COMP[raw[int(offs[i]):int(offs[i + 1])][::-1]] for i in range(n)])
        gm.tallies(reset=True)
        mats_r, inval_r, cnt_r = gm.match_reads(rc.tobytes(), offs, 0)
        expect_r = gm.tallies(reset=True)
        assert cnt_r.succ > 3000 and cnt_r.dp_reads > 500
        gm.memcpy(d_seq, rc.ctypes.data, len(rc), 1)
        gm.memcpy(d_mats, mats_r.ctypes.data, 8 * n, 1)
        gm.memcpy(d_inv, inval_r.ctypes.data, n, 1)
        for call in range(2):
            assert f(gm.h, d_seq, d_offs, d_mats, d_inv, n, 1, d_meth) == 0
            got = np.zeros(4 * ncpg, np.uint32)
            gm.memcpy(got.ctypes.data, d_meth, 16 * ncpg, 2)
            assert np.array_equal((got & 0xFFFF).astype(np.uint16).reshape(-1, 4), expect_r), "orient 1, call %d" % call
        # a read longer than FAME_MAX_READ_LEN is refused with FAME_ERR_READ
        long_offs = np.array([0, 300], np.uint64)
        gm.memcpy(d_offs, long_offs.ctypes.data, 16, 1)
        assert f(gm.h, d_seq, d_offs, d_mats, d_inv, 1, 0, d_meth) == -5
        assert b"FAME_MAX_READ_LEN" in lib().fame_gpu_last_error(gm.h)
        gm.memcpy(d_offs, offs.ctypes.data, 8 * (n + 1), 1)
        # the context stays usable
        m2, i2, c2 = gm.match_reads(seq, offs, FAME_MATCH_R1_FWD)
        assert np.array_equal(m2, mats) and np.array_equal(gm.tallies(reset=True), expect)
    finally:
        for p in bufs:
            gm.free(p)
        gm.close()
