"""The oracle (oracle/fame_oracle.c) against the reference's own outputs.

Every expected value here was produced by the compiled reference sources
(tests/golden/make_golden.py) or is a known-answer case of the reference's
LevenshtDP_unittest.cpp.
"""
import hashlib

import numpy as np

from oracle import oracle


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_lev_known_answers(kernels_golden):
    for c in kernels_golden["lev_kat"]:
        d, tr = oracle.lev(c["band"], c["row"], c["col"], c["col_end"], c["rev"], c["comp"])
        assert d == c["ref_dist"] == c["exp_dist"]
        assert tr == c["ref_trace"]
        if c["exp_trace"] is not None:
            assert tr == c["exp_trace"]


def test_lev_fame_comparators(kernels_golden):
    for c in kernels_golden["lev_fame"]:
        d, tr = oracle.lev(8, c["row"], c["col"], c["col_end"], c["rev"], c["comp"])
        assert (d, tr) == (c["ref_dist"], c["ref_trace"])


def test_shiftand(kernels_golden):
    nhit = 0
    for c in kernels_golden["shiftand"]:
        offs, errs = oracle.shiftand(c["pat"], c["text"], c["rev"])
        assert offs == c["offs"] and errs == c["errs"]
        nhit += len(offs)
    assert nhit > 100


def test_hopscotch_orders(kernels_golden):
    import ctypes as C
    L = oracle.lib()
    L.orc_hopscotch.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    for c in kernels_golden["hopscotch"]:
        keys = c["keys"]
        order = np.zeros(len(keys), np.uint32)
        fb = np.zeros(1, np.uint64)
        k = L.orc_hopscotch(keys.ctypes.data, len(keys), c["bucket_count"], order.ctypes.data, fb.ctypes.data)
        assert np.array_equal(order[:k], c["order"]) and int(fb[0]) == c["final_buckets"]


def test_index_build_matches_reference(golden, oracle_index):
    dig = golden["digests"].item()
    t = oracle_index.t
    for k in ("cpg_chrom", "cpg_pos", "cpgs_chrom", "cpgs_pos", "bucket_key", "bucket_start", "bucket_len",
              "kmer_meta", "strand", "win_start", "win_chrom", "win_sind", "win_eind", "filtered"):
        assert _digest(t[k]) == dig[k], k
    tm = t["kmer_tmask"].copy()
    tm[np.isin(t["kmer_meta"] & 0x7fffffff, golden["last_win"])] = 0
    assert _digest(tm) == dig["kmer_tmask_masked"]


def test_seed_order_matches_reference(golden, oracle_index):
    for c in golden["orders"]:
        f, r, bf, br = oracle_index.seed_order(c["seq"])
        assert np.array_equal(np.array(f, np.uint32).reshape(-1, 2), c["fwd"])
        assert np.array_equal(np.array(r, np.uint32).reshape(-1, 2), c["rev"])
        assert (bf, br) == (c["bf"], c["br"])


def test_matching_matches_reference(golden, oracle_index):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    for name, chunk, both in (("default", 0, False), ("chunk1000", 1000, False), ("both", 777, True)):
        o = oracle_index.match_se(seq, offs, chunk=chunk, both_strands=both)
        assert np.array_equal(o["invalid"], golden[name + "_invalid"]), name
        assert np.array_equal(o["mat"], golden[name + "_mat"]), name
        assert np.array_equal(o["meth"], golden[name + "_meth"]), name
        assert np.array_equal(o["counters"], golden[name + "_counters"]), name
    # the fixtures exercise every outcome
    c = golden["default_counters"]
    assert c[0] > 5000 and c[1] > 0 and c[2] > 0
    assert golden["default_meth"].astype(np.int64).sum() > 3000


PE_MODES = (("default", 0, False), ("chunk700", 700, False), ("both", 900, True))


def test_paired_matching_matches_reference(pe_golden, oracle_index):
    """matchPairedReads per chunk (queryRoutinePaired) on the paired fixture:
    per-mate matches, invalid flags, tallies and counters equal the reference's."""
    g = pe_golden
    s1, o1 = g["read_seq1"].tobytes(), g["read_offs1"]
    s2, o2 = g["read_seq2"].tobytes(), g["read_offs2"]
    for name, chunk, both in PE_MODES:
        r = oracle_index.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=both, maxpdist=int(g["maxpdist"]))
        for k in ("mat1", "mat2", "inv1", "inv2", "meth", "counters"):
            assert np.array_equal(r[k], g["%s_%s" % (name, k)]), (name, k)
