"""Generates the golden fixtures of the parity tests from the reference itself.

Run in a checkout that has the reference sources available to
oracle/build_ref.sh (it compiles them into oracle/_ref/libfame_ref.so):

    python tests/golden/make_golden.py

Writes tests/golden/se_small.npz (genome, reads, the reference's per-read
matches, CpG tallies and counters for three run modes, digests of its index
tables, and its hopscotch iteration orders for a set of reads) and
tests/golden/kernels.npz (LevenshtDP known-answer cases from
LevenshtDP_unittest.cpp plus random cases with FAME's comparators, ShiftAnd
cases, and hopscotch_map insertion orders), all computed by the compiled
reference code.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fame_gb300 import synth  # noqa: E402
from oracle import refbind  # noqa: E402

COMP = np.zeros(256, np.uint8)
for a, b in zip(b"ACGT", b"TGCA"):
    COMP[a] = b


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def small_workload():
    """Genome with repeats and N runs; reads with errors, both conversions and edge cases."""
    g = synth.make_genome([260_000, 140_000, 90_000], seed=101, repeat_frac=0.25, n_families=16,
                          fam_len=(300, 2500), divergence=(0.0, 0.06))
    g.seqs[1][40_000:40_400] = ord("N")
    g.seqs[1][90_000:90_012] = ord("N")
    g.seqs[2][1_000:1_003] = ord("N")
    rs = synth.make_reads(g, 6000, seed=102, sub_rate=0.015, indel_rate=0.003, repeat_read_frac=0.25)
    rng = np.random.default_rng(103)
    seqs, lens = rs.seqs.copy(), rs.lens.copy()
    lens[:40] = rng.integers(70, 100, 40)        # length gate (ReadQueue.cpp:430)
    seqs[40:50, 7] = ord("N")                    # N reads (ReadQueue.cpp:487)
    seqs[50:55, 3] = ord("a")                    # letters outside ACGTN
    for i in range(100, 1400):                   # G->A converted reads (reverse complement of a read)
        s = seqs[i, : lens[i]]
        seqs[i, : lens[i]] = COMP[s[::-1]]
    reads = [seqs[i, : lens[i]].tobytes() for i in range(len(lens))]
    # reads taken from the very start / end of chromosomes and around the N run
    for c, p in ((0, 0), (0, 3), (2, 0), (1, 40_350), (1, 140_000 - 100), (0, 260_000 - 101)):
        s = g.seqs[c][p:p + 100].copy()
        s[(s == ord("C"))] = ord("T")
        if ord("N") not in s:
            reads.append(s.tobytes())
    return g, reads


def kernel_cases(L: refbind.RefLib):
    rng = np.random.default_rng(7)
    out = {}
    # LevenshtDP_unittest.cpp (init_test 26-89, matching_test 92-246): inputs and expected results
    kat = [
        # band, row, col, col_end, rev, comp, expected dist, expected trace (None: not asserted there)
        (0, b"AG", b"CTAG", 3, 0, 0, 0, None), (0, b"AG", b"CCTCG", 4, 0, 0, 1, None),
        (1, b"AG", b"CTAG", 3, 0, 0, 0, None), (1, b"AG", b"CCTCG", 4, 0, 0, 1, None),
        (2, b"AG", b"CTAG", 3, 0, 0, 0, [0, 0]), (2, b"AG", b"CCTCG", 4, 0, 0, 1, [2, 0]),
        (2, b"AG", b"CCTCT", 4, 0, 0, 2, None),
        (2, b"ACTTTGACCG", b"AAACTGTGACTG", 11, 0, 0, 2, [0, 0, 0, 1, 0, 0, 0, 0, 1, 0]),
        (2, b"TCCAG", b"GACTGAA", 6, 1, 3, 1, [0, 0, 0, 1, 0]),
        (2, b"ACTAAGTGACTG", b"TTTTACTGTGACTG", 13, 0, 0, 2, [0, 0, 0, 2, 2, 0, 0, 0, 0, 0, 0, 0]),
        (2, b"TGTGACTT", b"TGTGACTAAT", 9, 0, 0, 2, [0, 0, 0, 0, 0, 0, 0, 3, 3, 0]),
        (2, b"ACGTGAACCTG", b"AAACGGTGAACTG", 12, 0, 0, 2, [0, 0, 0, 3, 0, 0, 0, 0, 0, 2, 0, 0]),
    ]
    kat_res = []
    for band, row, col, ce, rev, comp, ed, et in kat:
        d, tr = L.lev(band, row, col, ce, rev, comp)
        kat_res.append(dict(band=band, row=row, col=col, col_end=ce, rev=rev, comp=comp, exp_dist=ed,
                            exp_trace=et, ref_dist=d, ref_trace=tr))
    out["lev_kat"] = np.array(kat_res, dtype=object)
    # FAME comparators, band 8, random read/reference pairs with planted edits
    cases = []
    for i in range(300):
        n = int(rng.integers(80, 160))
        ref = synth.BASES[rng.integers(0, 4, n + 40)]
        read = ref[20:20 + n].copy()
        rev = int(i % 2)
        for _ in range(int(rng.integers(0, 7))):
            p = int(rng.integers(0, len(read)))
            k = rng.integers(0, 3)
            if k == 0:
                read[p] = synth.BASES[rng.integers(0, 4)]
            elif k == 1 and len(read) > 60:
                read = np.delete(read, p)
            else:
                read = np.insert(read, p, synth.BASES[rng.integers(0, 4)])
        if rev:
            read = COMP[read[::-1]]
        read[rng.random(len(read)) < 0.1] = ord("T")  # converted bases: T against C (or A/G) in the reference
        col = ref.tobytes()
        ce = int(20 + n - 1 + 2 + rng.integers(-2, 3))
        d, tr = L.lev(8, read.tobytes(), col, ce, rev, 2 if rev else 1)
        cases.append(dict(row=read.tobytes(), col=col, col_end=ce, rev=rev, comp=2 if rev else 1, ref_dist=d,
                          ref_trace=tr))
    out["lev_fame"] = np.array(cases, dtype=object)
    # ShiftAnd (querySeq / queryRevSeq) on texts with planted approximate occurrences
    sa = []
    for i in range(300):
        m = int(rng.integers(80, 151))
        pat = synth.BASES[rng.integers(0, 4, m)]
        text = synth.BASES[rng.integers(0, 4, int(rng.integers(300, 2100)))]
        for _ in range(int(rng.integers(0, 4))):
            p = int(rng.integers(0, max(1, len(text) - m)))
            occ = pat.copy()
            for _ in range(int(rng.integers(0, 8))):
                q = int(rng.integers(0, m))
                occ[q] = synth.BASES[rng.integers(0, 4)]
            occ[(occ == ord("T")) & (rng.random(m) < 0.5)] = ord("C")
            text[p:p + m] = occ[: len(text) - p]
        if i % 5 == 0:
            text[rng.integers(0, len(text), 3)] = ord("N")
        rev = int(i % 2)
        tb = (COMP[text[::-1]] if rev else text).tobytes()
        tb = bytes(b if b in b"ACGT" else ord("N") for b in tb) if rev else tb
        offs, errs = L.shiftand(pat.tobytes(), tb, rev)
        sa.append(dict(pat=pat.tobytes(), text=tb, rev=rev, offs=offs, errs=errs))
    out["shiftand"] = np.array(sa, dtype=object)
    # tsl::hopscotch_map iteration orders for adversarial key sequences
    import ctypes as C
    F = L.lib.fame_ref_hopscotch
    F.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p]
    hs = []
    for t in range(400):
        kind = t % 5
        n = int(rng.integers(1, 300))
        bc = int(rng.integers(0, 64))
        if kind == 0:
            keys = rng.integers(0, 1 << 20, n)
        elif kind == 1:
            keys = rng.integers(0, 8, n) * 64 + rng.integers(0, 3, n)
        elif kind == 2:
            keys = np.arange(n) * int(rng.choice([16, 32, 64, 128]))
        elif kind == 3:
            keys = rng.integers(0, 4, n) * 1024 + rng.integers(0, 70, n)
        else:
            keys = np.concatenate([np.arange(100) * 512, rng.integers(0, 50, n)])
        keys = keys.astype(np.uint32)
        order = np.zeros(len(keys), np.uint32)
        fb = np.zeros(1, np.uint64)
        k = F(keys.ctypes.data, len(keys), bc, order.ctypes.data, fb.ctypes.data)
        hs.append(dict(keys=keys, bucket_count=bc, order=order[:k].copy(), final_buckets=int(fb[0])))
    out["hopscotch"] = np.array(hs, dtype=object)
    return out


def main():
    L = refbind.RefLib()
    assert L.readlen == 100, "fixtures are for READLEN 100"
    g, reads = small_workload()
    fasta = "/tmp/fame_golden_genome.fa"
    g.write_fasta(fasta)
    ri = L.build(fasta)
    d = ri.dump()
    # the reference reads past the chromosome end for the T masks of the last
    # window of a chromosome (RefGenome.h:62-100): exclude those entries
    last_win = np.array([np.nonzero(d["win_chrom"] == c)[0].max() for c in range(len(g.seqs))])
    tm = d["kmer_tmask"].copy()
    tm[np.isin(d["kmer_meta"] & 0x7fffffff, last_win)] = 0
    digests = {k: digest(v) for k, v in d.items() if k != "kmer_tmask"}
    digests["kmer_tmask_masked"] = digest(tm)
    seq = b"".join(reads)
    offs = np.zeros(len(reads) + 1, np.uint64)
    np.cumsum([len(r) for r in reads], out=offs[1:])
    runs = {}
    for name, chunk, both in (("default", 0, False), ("chunk1000", 1000, False), ("both", 777, True)):
        r = ri.match_se(seq, offs, chunk=chunk, both_strands=both)
        runs[name] = r
    orders = []
    for i in range(0, len(reads), 20):
        s = reads[i]
        if len(s) < 80 or b"N" in s:
            continue
        for s2 in (s, bytes(COMP[np.frombuffer(s, np.uint8)[::-1]])):
            if 0 in s2:
                continue
            f, rv, bf, br = ri.seed_order(s2)
            orders.append(dict(seq=s2, fwd=np.array(f, np.uint32).reshape(-1, 2), rev=np.array(rv, np.uint32).reshape(-1, 2),
                               bf=bf, br=br))
    np.savez_compressed(
        os.path.join(HERE, "se_small.npz"),
        chrom_lens=np.array([len(s) for s in g.seqs], np.int64),
        genome=np.concatenate(g.seqs),
        read_seq=np.frombuffer(seq, np.uint8), read_offs=offs,
        digests=np.array(digests, dtype=object),
        n_tables=np.array([len(d[k]) for k in ("cpg_pos", "cpgs_pos", "bucket_key", "kmer_meta", "win_start", "filtered")]),
        **{"%s_%s" % (name, k): v for name, r in runs.items() for k, v in r.items() if k != "seconds"},
        orders=np.array(orders, dtype=object),
        last_win=last_win,
    )
    ri.close()
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), **kernel_cases(L))
    print("golden fixtures written; default counters", runs["default"]["counters"])


if __name__ == "__main__":
    main()
