"""Generates the paired-end golden fixture from the reference itself.

Run in a checkout that has the reference sources available to
oracle/build_ref.sh (compiled with MAXPDIST 550, its CONST.h value):

    python tests/golden/make_golden_pe.py

Writes tests/golden/pe_small.npz: read pairs on the genome of se_small.npz
(the same seeded workload), and for three run modes the reference's per-mate
matches, invalid flags, CpG tallies and matchPairedReads counters
{succ, nonUnique, unSucc, succPaired, tooShort, r1Fwd, r1Rev, matchR1Fwd};
matches of both mates of a pair with an invalid mate are stored as 0 (the
reference leaves them stale).
Pairs whose fragment lies in the last 4.2 kbp of a chromosome are left out:
there the reference builds the T masks of the chromosome's last window from
bytes past the chromosome end (RefGenome.h:62-100), which no other build can
reproduce.  The script checks that the oracle, on its own index, agrees.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from fame_gb300 import synth  # noqa: E402
from make_golden import COMP, small_workload  # noqa: E402
from oracle import refbind  # noqa: E402
from oracle.oracle import OracleIndex  # noqa: E402

MAXPDIST = 550
MODES = (("default", 0, False), ("chunk700", 700, False), ("both", 900, True))


def pairs_workload(g):
    rng = np.random.default_rng(211)
    sets = [synth.make_pairs(g, 2600, seed=212, sub_rate=0.015, indel_rate=0.003),
            synth.make_pairs(g, 500, seed=213, read_len=150, inner=(20, 300), sub_rate=0.01, indel_rate=0.002)]
    m1, m2 = [], []
    for r1, r2 in sets:
        for i in range(len(r1)):
            L = len(g.seqs[r1.chrom[i]])
            if r1.start[i] + 700 > L - 4200:
                continue
            m1.append(r1.seqs[i, : r1.lens[i]].copy())
            m2.append(r2.seqs[i, : r2.lens[i]].copy())
    n = len(m1)
    for i in range(0, 20):
        m1[i] = m1[i][: int(rng.integers(60, 75))]          # mate 1 below ceil(0.75 * READLEN)
    for i in range(20, 30):
        m2[i][5] = ord("N")                                    # N in mate 2
    for i in range(30, 35):
        m1[i][9] = ord("a")                                    # letter outside ACGT
    for i in range(35, 70):
        m1[i] = m1[i][: int(rng.integers(75, 100))]           # uneven mate lengths
    for i in range(70, 90):                                    # discordant: mate 2 from another pair
        j = int(rng.integers(200, n))
        m2[i] = m2[j].copy()
    for i in range(90, 110):                                   # mates swapped (the other orientation)
        m1[i], m2[i] = m2[i], m1[i]
    for i in range(110, 130):                                  # mate 2 reverse-complemented (same strand)
        m2[i] = COMP[m2[i][::-1]]
    order = rng.permutation(n)
    m1 = [m1[i] for i in order]
    m2 = [m2[i] for i in order]
    pack = []
    for mates in (m1, m2):
        offs = np.zeros(n + 1, np.uint64)
        np.cumsum([len(x) for x in mates], out=offs[1:])
        pack.append((b"".join(x.tobytes() for x in mates), offs))
    return pack


def main():
    L = refbind.RefLib()
    assert L.readlen == 100, "fixtures are for READLEN 100"
    g, _ = small_workload()
    fasta = "/tmp/fame_golden_genome.fa"
    g.write_fasta(fasta)
    (s1, o1), (s2, o2) = pairs_workload(g)
    ri = L.build(fasta)
    oi = OracleIndex.build(g.seqs, readlen=100)
    out = dict(read_seq1=np.frombuffer(s1, np.uint8), read_offs1=o1, read_seq2=np.frombuffer(s2, np.uint8),
               read_offs2=o2, maxpdist=np.array(MAXPDIST))
    for name, chunk, both in MODES:
        r = ri.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=both)
        # the reference leaves Read::mat as it was (stale buffer contents) for
        # both mates of a pair with an invalid mate; only pairs it matched
        # carry matches
        bad = (r["inv1"] != 0) | (r["inv2"] != 0)
        r["mat1"][bad] = 0
        r["mat2"][bad] = 0
        o = oi.match_pe(s1, o1, s2, o2, chunk=chunk, both_strands=both, maxpdist=MAXPDIST)
        for k in ("mat1", "mat2", "inv1", "inv2", "meth", "counters"):
            assert np.array_equal(r[k], o[k]), "oracle disagrees with the reference on %s (%s)" % (k, name)
            out["%s_%s" % (name, k)] = r[k]
        print(name, "counters", r["counters"])
    ri.close()
    np.savez_compressed(os.path.join(HERE, "pe_small.npz"), **out)
    print("pe_small.npz written:", len(o1) - 1, "pairs")


if __name__ == "__main__":
    main()
