"""Seeded synthetic whole-genome-bisulfite workloads.

FAME is benchmarked on synthetic genomes and bisulfite reads (there is no
public dataset bundled with it, and its own simulator needs a real FASTA and
``std::random_device``).  This module generates, from a fixed seed and with
numpy's PCG64 generator (bit-identical on x86 and Arm):

* a genome: i.i.d. bases with a given composition, interspersed repeat
  families pasted in at a given divergence, CpG dinucleotides thinned to a
  target density, and a methylation state per CpG site;
* single-end reads: uniform start, 50/50 genome strand, bisulfite conversion
  (every C that is not a methylated CpG C becomes T on the read's strand),
  substitutions and 1-bp indels, optional trimmed-length distribution.

Everything is uppercase ASCII (``A C G T``) held in numpy ``uint8`` arrays.
"""
from __future__ import annotations

import dataclasses
import numpy as np

A, C, G, T, N = 65, 67, 71, 84, 78
BASES = np.array([A, C, G, T], dtype=np.uint8)

_COMP = np.arange(256, dtype=np.uint8)
for _a, _b in ((A, T), (C, G), (G, C), (T, A), (N, N)):
    _COMP[_a] = _b

_IDX = np.full(256, 255, dtype=np.uint8)
for _i, _b in enumerate((A, C, G, T)):
    _IDX[_b] = _i


@dataclasses.dataclass
class Genome:
    names: list
    seqs: list            # list of uint8 arrays (ASCII)
    meth: list            # list of bool arrays: True at both bases of a methylated CpG
    repeat_copies: list   # list of (chrom, start, length) of pasted repeat copies

    @property
    def total_len(self) -> int:
        return int(sum(len(s) for s in self.seqs))

    def write_fasta(self, path: str, width: int = 80) -> None:
        with open(path, "wb") as f:
            for name, s in zip(self.names, self.seqs):
                f.write(b">" + name.encode() + b"\n")
                b = s.tobytes()
                for i in range(0, len(b), width):
                    f.write(b[i:i + width] + b"\n")


@dataclasses.dataclass
class ReadSet:
    seqs: np.ndarray      # (n, max_len) uint8, ASCII, zero padded
    lens: np.ndarray      # (n,) int32
    chrom: np.ndarray     # truth: chromosome index
    start: np.ndarray     # truth: leftmost forward-strand position of the source fragment
    fwd: np.ndarray       # truth: True if sampled from the forward genome strand

    def __len__(self) -> int:
        return int(self.lens.shape[0])

    def concat(self):
        """Return (bytes of all sequences back to back, uint64 offsets[n+1])."""
        lens = self.lens.astype(np.int64)
        offs = np.zeros(len(lens) + 1, dtype=np.uint64)
        np.cumsum(lens, out=offs[1:])
        mask = np.arange(self.seqs.shape[1])[None, :] < lens[:, None]
        return self.seqs[mask].tobytes(), offs

    def subset(self, idx) -> "ReadSet":
        return ReadSet(self.seqs[idx], self.lens[idx], self.chrom[idx], self.start[idx], self.fwd[idx])

    def write_fastq(self, path: str, block: int = 500_000) -> None:
        """Records "@r<i>" / sequence / "+" / all-'I' qualities; reads of one
        length are written as fixed-width blocks (names "@r"), others one by one."""
        lens = self.lens
        if len(self) and (lens == lens[0]).all():
            L = int(lens[0])
            with open(path, "wb") as f:
                for b0 in range(0, len(self), block):
                    s = self.seqs[b0:b0 + block, :L]
                    rec = np.empty((len(s), 2 * L + 7), np.uint8)
                    rec[:, :3] = np.frombuffer(b"@r\n", np.uint8)
                    rec[:, 3:3 + L] = s
                    rec[:, 3 + L:6 + L] = np.frombuffer(b"\n+\n", np.uint8)
                    rec[:, 6 + L:6 + 2 * L] = ord("I")
                    rec[:, -1] = ord("\n")
                    f.write(rec.tobytes())
            return
        with open(path, "wb") as f:
            for i in range(len(self)):
                s = self.seqs[i, : self.lens[i]].tobytes()
                f.write(b"@r%d\n%s\n+\n%s\n" % (i, s, b"I" * len(s)))


def _random_bases(rng, n, base_p):
    # exact per-mille composition through a lookup table (fast, platform independent)
    counts = np.round(np.asarray(base_p) * 1000).astype(int)
    lut = np.repeat(BASES, counts)
    return lut[rng.integers(0, len(lut), size=n, dtype=np.int32)]


def make_genome(chrom_lengths, seed, base_p=(0.295, 0.205, 0.205, 0.295), cpg_frac=0.01,
                meth_p=0.7, repeat_frac=0.0, n_families=2000, fam_len=(300, 6000),
                divergence=(0.10, 0.20), names=None) -> Genome:
    rng = np.random.default_rng(seed)
    seqs = [_random_bases(rng, int(L), base_p) for L in chrom_lengths]
    total = sum(len(s) for s in seqs)
    copies = []
    if repeat_frac > 0:
        lo, hi = np.log(fam_len[0]), np.log(fam_len[1])
        fam_lens = np.exp(rng.uniform(lo, hi, size=n_families)).astype(np.int64)
        fams = [_random_bases(rng, int(L), base_p) for L in fam_lens]
        weights = np.array([len(s) for s in seqs], dtype=np.float64)
        weights /= weights.sum()
        target = int(repeat_frac * total)
        placed = 0
        while placed < target:
            f = int(rng.integers(0, n_families))
            src = fams[f]
            d = rng.uniform(divergence[0], divergence[1])
            cp = src.copy()
            mut = rng.random(len(cp)) < d
            nm = int(mut.sum())
            if nm:
                cp[mut] = BASES[(_IDX[cp[mut]] + rng.integers(1, 4, size=nm)) % 4]
            if rng.random() < 0.5:
                cp = _COMP[cp[::-1]]
            ci = int(rng.choice(len(seqs), p=weights))
            L = len(seqs[ci])
            if L <= len(cp):
                continue
            st = int(rng.integers(0, L - len(cp)))
            seqs[ci][st:st + len(cp)] = cp
            copies.append((ci, st, len(cp)))
            placed += len(cp)
    meth = []
    for s in seqs:
        is_cg = (s[:-1] == C) & (s[1:] == G)
        pos = np.nonzero(is_cg)[0]
        frac = len(pos) / max(1, len(s))
        keep_p = min(1.0, cpg_frac / frac) if frac > 0 else 1.0
        keep = rng.random(len(pos)) < keep_p
        drop = pos[~keep]
        s[drop + 1] = np.where(rng.random(len(drop)) < 0.5, A, T).astype(np.uint8)
        kept = pos[keep]
        m = np.zeros(len(s), dtype=bool)
        mk = kept[rng.random(len(kept)) < meth_p]
        m[mk] = True
        m[mk + 1] = True
        meth.append(m)
    if names is None:
        names = ["chr%d" % (i + 1) for i in range(len(seqs))]
    return Genome(list(names), seqs, meth, copies)


def _bisulfite(genome: Genome):
    """Per chromosome: forward strand after conversion, and the forward-coordinate
    image of the converted reverse strand (G->A unless a methylated CpG G)."""
    conv_f, conv_r = [], []
    for s, m in zip(genome.seqs, genome.meth):
        cf = s.copy()
        cf[(s == C) & ~m] = T
        cr = s.copy()
        cr[(s == G) & ~m] = A
        conv_f.append(cf)
        conv_r.append(cr)
    return conv_f, conv_r


def make_reads(genome: Genome, n_reads, seed, read_len=100, sub_rate=0.005, indel_rate=0.0005,
               length_sampler=None, error_sampler=None, repeat_read_frac=0.0, batch=500_000) -> ReadSet:
    """Single-end bisulfite reads.

    length_sampler(rng, n) -> int array of read lengths (default: all read_len).
    error_sampler(rng, n) -> float array of per-read substitution rates (default: sub_rate);
    indels then occur at indel_rate/sub_rate times that rate.
    repeat_read_frac: fraction of reads whose start is drawn inside a pasted repeat copy.
    """
    rng = np.random.default_rng(seed)
    conv_f, conv_r = _bisulfite(genome)
    nchr = len(genome.seqs)
    clen = np.array([len(s) for s in genome.seqs], dtype=np.int64)
    pad = 8
    lens = (np.full(n_reads, read_len, dtype=np.int32) if length_sampler is None
            else np.asarray(length_sampler(rng, n_reads), dtype=np.int32))
    maxL = int(lens.max()) if n_reads else read_len
    W = maxL + pad
    chrom = rng.choice(nchr, size=n_reads, p=clen / clen.sum())
    start = (rng.random(n_reads) * (clen[chrom] - W)).astype(np.int64)
    if repeat_read_frac > 0 and genome.repeat_copies:
        rr = rng.random(n_reads) < repeat_read_frac
        cps = np.array(genome.repeat_copies, dtype=np.int64)
        pick = cps[rng.integers(0, len(cps), size=int(rr.sum()))]
        off = (rng.random(len(pick)) * np.maximum(1, pick[:, 2] - maxL)).astype(np.int64)
        chrom[rr] = pick[:, 0]
        start[rr] = np.minimum(pick[:, 1] + off, clen[pick[:, 0]] - W)
    fwd = rng.random(n_reads) < 0.5
    rates = (np.full(n_reads, sub_rate) if error_sampler is None
             else np.asarray(error_sampler(rng, n_reads), dtype=np.float64))
    irates = rates * (indel_rate / sub_rate if sub_rate > 0 else 0.0)
    out = np.zeros((n_reads, maxL), dtype=np.uint8)
    for b0 in range(0, n_reads, batch):
        b1 = min(n_reads, b0 + batch)
        nb = b1 - b0
        frag = np.empty((nb, W), dtype=np.uint8)
        cols = np.arange(W)
        for ci in range(nchr):
            sel = np.nonzero(chrom[b0:b1] == ci)[0]
            if len(sel) == 0:
                continue
            idx = start[b0:b1][sel, None] + cols[None, :]
            f_ok = fwd[b0:b1][sel]
            frag[sel[f_ok]] = conv_f[ci][idx[f_ok]]
            frag[sel[~f_ok]] = _COMP[conv_r[ci][idx[~f_ok]][:, ::-1]]
        # substitutions
        sub = rng.random((nb, W)) < rates[b0:b1, None]
        ns = int(sub.sum())
        if ns:
            frag[sub] = BASES[(_IDX[frag[sub]] + rng.integers(1, 4, size=ns)) % 4]
        # 1-bp indels (applied one event per pass; reads with several events take several passes)
        nev = rng.binomial(maxL, np.minimum(1.0, irates[b0:b1]))
        for _ in range(int(nev.max()) if nb else 0):
            rows = np.nonzero(nev > 0)[0]
            nev[rows] -= 1
            p = rng.integers(0, maxL, size=len(rows))
            ins = rng.random(len(rows)) < 0.5
            j = np.arange(W)[None, :]
            src = np.where(j < p[:, None], j, np.where(ins[:, None], j - 1, j + 1))
            src = np.clip(src, 0, W - 1)
            new = np.take_along_axis(frag[rows], src, axis=1)
            ib = rows[ins]
            new[ins, p[ins]] = BASES[rng.integers(0, 4, size=len(ib))]
            frag[rows] = new
        out[b0:b1] = frag[:, :maxL]
    col = np.arange(maxL)[None, :]
    out[col >= lens[:, None]] = 0
    return ReadSet(out, lens, chrom.astype(np.int32), start, fwd)


# --- the five workloads FAME is measured on (sizes as stated per workload) ---

def _uneven_len(rng, n):
    full = rng.random(n) < 0.6
    return np.where(full, 150, rng.integers(36, 150, size=n))


def _per_read_err(rng, n):
    return rng.uniform(0.005, 0.02, size=n)


def _mammal_lengths(n=24, total=3_000_000_000):
    w = np.linspace(250, 50, n)
    return [int(x) for x in (w / w.sum() * total)]


WORKLOADS = {
    # 4 x 5 Mbp, 100k SE 100 bp, 0.5% subs / 0.05% indels, seed 1
    "se100_20mbp": dict(genome=dict(chrom_lengths=[5_000_000] * 4, seed=1, meth_p=0.7),
                        reads=dict(n_reads=100_000, seed=2, sub_rate=0.005, indel_rate=0.0005)),
    # 8 chromosomes / 300 Mbp, 8% repeats, 5M SE 100 bp, 1% subs / 0.1% indels
    "se100_300mbp": dict(genome=dict(chrom_lengths=[37_500_000] * 8, seed=11, meth_p=0.7,
                                     repeat_frac=0.08),
                         reads=dict(n_reads=5_000_000, seed=12, sub_rate=0.01, indel_rate=0.001)),
    # the 300 Mbp genome above; single-cell jobs: Poisson arrivals at 20 jobs/s, log-normal read counts
    # (median 200k, clipped to [2k, 2M]), SE 100 bp
    "sc_serving": dict(genome=dict(chrom_lengths=[37_500_000] * 8, seed=11, meth_p=0.7, repeat_frac=0.08),
                       jobs=dict(n_jobs=24, rate=20.0, median=200_000, sigma=1.0, lo=2_000, hi=2_000_000, seed=14,
                                 sub_rate=0.01, indel_rate=0.001)),
    # the 300 Mbp genome above, 1.5M pairs of 2 x 100 bp, inner distance U[20, 400]
    "pe100_300mbp": dict(genome=dict(chrom_lengths=[37_500_000] * 8, seed=11, meth_p=0.7, repeat_frac=0.08),
                         pairs=dict(n_pairs=1_500_000, seed=13, inner=(20, 400), sub_rate=0.01, indel_rate=0.001)),
    # 24 chromosomes / 3.0 Gbp, 45% repeats, READLEN 150 uneven trimmed reads
    "se150_uneven_3gbp": dict(genome=dict(chrom_lengths=_mammal_lengths(), seed=21, meth_p=0.75,
                                          repeat_frac=0.45),
                              reads=dict(n_reads=20_000_000, seed=22, read_len=150,
                                         length_sampler=_uneven_len, error_sampler=_per_read_err,
                                         sub_rate=0.01, indel_rate=0.001, repeat_read_frac=0.05)),
}


def make_pairs(genome: Genome, n_pairs, seed, read_len=100, inner=(20, 400), sub_rate=0.01, indel_rate=0.001):
    """Paired-end bisulfite reads: a fragment of read_len + inner + read_len bases
    (inner uniform in the closed range) from a random strand; mate 1 is the
    fragment's first read_len bases, mate 2 the reverse complement of its last
    read_len bases (the opposite strand).  Errors are drawn per mate."""
    rng = np.random.default_rng(seed)

    def frag_len(r, n):
        return read_len + r.integers(inner[0], inner[1] + 1, size=n) + read_len

    fr = make_reads(genome, n_pairs, seed=int(rng.integers(1 << 31)), read_len=read_len + inner[1] + read_len,
                    length_sampler=frag_len, sub_rate=0.0, indel_rate=0.0)
    m1 = np.zeros((n_pairs, read_len), np.uint8)
    m2 = np.zeros((n_pairs, read_len), np.uint8)
    for i in range(n_pairs):
        f = fr.seqs[i, : fr.lens[i]]
        m1[i] = f[:read_len]
        m2[i] = _COMP[f[-read_len:][::-1]]
    lens = np.full(n_pairs, read_len, np.int32)

    def errs(mat):
        out = mat.copy()
        sub = rng.random(out.shape) < sub_rate
        ns = int(sub.sum())
        if ns:
            out[sub] = BASES[(_IDX[out[sub]] + rng.integers(1, 4, size=ns)) % 4]
        for i in np.nonzero(rng.random(n_pairs) < indel_rate * read_len)[0]:
            p = int(rng.integers(0, read_len))
            row = list(out[i])
            if rng.random() < 0.5:
                del row[p]
                row.append(int(BASES[rng.integers(0, 4)]))
            else:
                row.insert(p, int(BASES[rng.integers(0, 4)]))
                row = row[:read_len]
            out[i] = np.array(row, np.uint8)
        return out

    r1 = ReadSet(errs(m1), lens.copy(), fr.chrom, fr.start, fr.fwd)
    r2 = ReadSet(errs(m2), lens.copy(), fr.chrom, fr.start, ~fr.fwd)
    return r1, r2
