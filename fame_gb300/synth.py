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
        """Records "@r" / sequence / "+" / all-'I' qualities (FAME reads the
        sequence line only), written in blocks."""
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
            # reads of different lengths: records laid out with offsets, in blocks
            for b0 in range(0, len(self), block):
                L = lens[b0:b0 + block].astype(np.int64)
                rl = 2 * L + 7
                start = np.zeros(len(L) + 1, np.int64)
                np.cumsum(rl, out=start[1:])
                rec = np.full(int(start[-1]), ord("I"), np.uint8)
                st = start[:-1]
                rec[st] = ord("@")
                rec[st + 1] = ord("r")
                rec[st + 2] = ord("\n")
                for k, ch in ((3, "\n"), (4, "+"), (5, "\n")):
                    rec[st + L + k] = ord(ch)
                rec[start[1:] - 1] = ord("\n")
                cols = np.arange(self.seqs.shape[1])[None, :]
                m = cols < L[:, None]
                pos = (st[:, None] + 3 + cols)[m]
                rec[pos] = self.seqs[b0:b0 + block][m]
                f.write(rec.tobytes())


def bgzf_compress(src: str, dst: str, level: int = 1, block: int = 65280, threads: int = 0) -> None:
    """Writes src as BGZF (the blocked gzip of bgzip: members of at most
    64 KiB, each with a 'BC' extra subfield holding its size, then the empty
    end-of-file member); members compressed on host threads."""
    import os
    import struct
    import zlib
    from concurrent.futures import ThreadPoolExecutor

    def member(data: bytes) -> bytes:
        co = zlib.compressobj(level, zlib.DEFLATED, -15)
        cdata = co.compress(data) + co.flush()
        head = struct.pack("<BBBBIBBHBBHH", 31, 139, 8, 4, 0, 0, 255, 6, ord("B"), ord("C"), 2, 18 + len(cdata) + 7)
        return head + cdata + struct.pack("<II", zlib.crc32(data) & 0xFFFFFFFF, len(data))

    with open(src, "rb") as f, open(dst, "wb") as g, ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
        while True:
            piece = f.read(block * 1024)
            if not piece:
                break
            for m in ex.map(member, [piece[i:i + block] for i in range(0, len(piece), block)]):
                g.write(m)
        g.write(member(b""))


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
    # 24 chromosomes / 3.0 Gbp (250 Mbp down to 50 Mbp), 45% repeats, methylation 0.75; READLEN 150:
    # 20M SE reads, 60% at 150 bp and 40% uniform in 36-149 bp, 0.5-2% errors per read (a tenth of them
    # 1-bp indels), 5% of the reads drawn from repeat copies
    "se150_uneven_3gbp": dict(large=True,
                              genome=dict(chrom_lengths=_mammal_lengths(), seed=21, meth_p=0.75,
                                          repeat_frac=0.45),
                              reads=dict(n_reads=20_000_000, seed=22, read_len=150,
                                         length_sampler=_uneven_len, error_sampler=_per_read_err,
                                         sub_rate=0.01, indel_rate=0.001, repeat_read_frac=0.05)),
    # the 3 Gbp workload's models on a 30 Mbp genome (4 chromosomes) with 1.2M reads: quick checks
    "se150_uneven_30mbp": dict(large=True,
                               genome=dict(chrom_lengths=[10_000_000, 8_000_000, 7_000_000, 5_000_000], seed=31,
                                           meth_p=0.75, repeat_frac=0.45),
                               reads=dict(n_reads=1_200_000, seed=32, read_len=150,
                                          length_sampler=_uneven_len, error_sampler=_per_read_err,
                                          sub_rate=0.01, indel_rate=0.001, repeat_read_frac=0.05)),
    "pe100_30mbp": dict(large=True, maxpdist=400,
                        genome=dict(chrom_lengths=[10_000_000, 8_000_000, 7_000_000, 5_000_000], seed=31,
                                    meth_p=0.75, repeat_frac=0.45),
                        pairs=dict(n_pairs=1_200_000, seed=33, inner=(20, 400), sub_rate=0.01, indel_rate=0.001)),
    # the 3 Gbp genome above; single-cell jobs of SE 100 bp reads (READLEN 100): Poisson arrivals at 20
    # jobs/s, log-normal read counts (median 200k, clipped to [2k, 2M]), each cell with its own CpG
    # methylation probability drawn from Beta(6, 2)
    "sc_serving_3gbp": dict(large=True,
                            genome=dict(chrom_lengths=_mammal_lengths(), seed=21, meth_p=0.75, repeat_frac=0.45),
                            jobs=dict(n_jobs=24, rate=20.0, median=200_000, sigma=1.0, lo=2_000, hi=2_000_000,
                                      seed=24, sub_rate=0.01, indel_rate=0.001, cell_beta=(6.0, 2.0))),
    # the 3 Gbp genome above; 20M pairs of 2 x 100 bp, inner distance U[20, 400], mate on the opposite
    # strand, 1% substitutions / 0.1% indels; MAXPDIST 400
    "pe100_3gbp": dict(large=True, maxpdist=400,
                       genome=dict(chrom_lengths=_mammal_lengths(), seed=21, meth_p=0.75, repeat_frac=0.45),
                       pairs=dict(n_pairs=20_000_000, seed=23, inner=(20, 400), sub_rate=0.01, indel_rate=0.001)),
}


def genome_of(name, threads=0):
    """The workload's genome (genome-scale generator for the 3 Gbp workloads)."""
    spec = WORKLOADS[name]
    if spec.get("large"):
        return make_genome_large(**spec["genome"], threads=threads)
    return make_genome(**spec["genome"])


def reads_of(name, genome, n_reads=0, threads=0):
    """(ReadSet, READLEN) of a single-end workload; n_reads overrides the count."""
    spec = WORKLOADS[name]
    rk = dict(spec["reads"])
    if n_reads:
        rk["n_reads"] = n_reads
    if spec.get("large"):
        return make_reads_large(genome, **rk, threads=threads), rk.get("read_len", 100)
    return make_reads(genome, **rk), rk.get("read_len", 100)


def pairs_of(name, genome, n_pairs=0, threads=0):
    """(mate 1 ReadSet, mate 2 ReadSet) of a paired-end workload."""
    spec = WORKLOADS[name]
    pk = dict(spec["pairs"])
    if n_pairs:
        pk["n_pairs"] = n_pairs
    if spec.get("large"):
        return make_pairs_large(genome, **pk, threads=threads)
    return make_pairs(genome, **pk)


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


# --- genome-scale generators (3 Gbp workloads) --------------------------------
#
# The same models as make_genome / make_reads, restated for multi-gigabase
# inputs: every per-base step is a vectorised numpy operation (numpy's bulk
# random fills and array ops release the GIL), chromosomes and read batches
# run on a thread pool, and each chromosome / read batch draws from its own
# PCG64 stream spawned from the seed, so the output does not depend on the
# thread count.  Methylation is kept as sorted positions of methylated CpG Cs
# per chromosome instead of a per-base mask, and bisulfite conversion is
# applied per read fragment.

def _threads(n=0):
    import os
    return n if n > 0 else max(1, min(32, os.cpu_count() or 1))


def _base_lut(base_p):
    # 65536-entry table with the composition to 1/65536
    counts = np.floor(np.asarray(base_p, dtype=np.float64) * 65536).astype(np.int64)
    counts[np.argmax(counts)] += 65536 - counts.sum()
    return np.repeat(BASES, counts)


def _fast_bases(rng, n, lut):
    return lut[rng.integers(0, 65536, size=n, dtype=np.uint16)]


@dataclasses.dataclass
class LargeGenome:
    names: list
    seqs: list            # list of uint8 arrays (ASCII)
    meth_pos: list        # per chromosome: sorted int64 positions of the C of each methylated CpG
    cpg_pos: list         # per chromosome: sorted int64 positions of the C of every CpG
    repeat_copies: np.ndarray   # (k, 3) int64: chrom, start, length

    @property
    def total_len(self) -> int:
        return int(sum(len(s) for s in self.seqs))

    def write_fasta(self, path: str, width: int = 80) -> None:
        Genome.write_fasta(self, path, width)


def make_genome_large(chrom_lengths, seed, base_p=(0.295, 0.205, 0.205, 0.295), cpg_frac=0.01, meth_p=0.75,
                      repeat_frac=0.45, n_families=2000, fam_len=(300, 6000), divergence=(0.10, 0.20),
                      names=None, threads=0) -> LargeGenome:
    """i.i.d. bases, repeat copies pasted at `repeat_frac` of each chromosome
    (families of log-uniform length, per-copy divergence, either strand), CpGs
    thinned to `cpg_frac` of positions, each kept CpG methylated with `meth_p`."""
    import concurrent.futures as cf
    lut = _base_lut(base_p)
    nchr = len(chrom_lengths)
    kids = np.random.SeedSequence(seed).spawn(nchr + 1)
    frng = np.random.default_rng(kids[-1])
    lo, hi = np.log(fam_len[0]), np.log(fam_len[1])
    flen = np.exp(frng.uniform(lo, hi, size=n_families)).astype(np.int64)
    foff = np.zeros(n_families + 1, np.int64)
    np.cumsum(flen, out=foff[1:])
    fcat = _fast_bases(frng, int(foff[-1]), lut)
    mean_len = float(flen.mean())

    def one(ci):
        rng = np.random.default_rng(kids[ci])
        L = int(chrom_lengths[ci])
        s = _fast_bases(rng, L, lut)
        copies = np.zeros((0, 3), np.int64)
        if repeat_frac > 0:
            target = repeat_frac * L
            k = int(target / mean_len * 1.3) + 16
            f = rng.integers(0, n_families, size=k)
            ln = flen[f]
            keep = np.searchsorted(np.cumsum(ln), target) + 1
            f, ln = f[:keep], ln[:keep]
            ok = ln < L
            f, ln = f[ok], ln[ok]
            k = len(f)
            st = (rng.random(k) * (L - ln)).astype(np.int64)
            flip = rng.random(k) < 0.5
            div = rng.uniform(divergence[0], divergence[1], size=k)
            copies = np.stack([np.full(k, ci, np.int64), st, ln], axis=1)
            i = 0
            while i < k:   # sub-batches of about 8M copied bases
                j = min(k, i + max(1, int(8e6 // mean_len)))
                lb = ln[i:j]
                tot = int(lb.sum())
                cstart = np.zeros(j - i, np.int64)
                np.cumsum(lb[:-1], out=cstart[1:])
                rep = np.repeat(np.arange(j - i), lb)
                pos = np.arange(tot, dtype=np.int64) - cstart[rep]
                fl = flip[i:j][rep]
                src = np.where(fl, foff[f[i:j]][rep] + lb[rep] - 1 - pos, foff[f[i:j]][rep] + pos)
                b = fcat[src]
                b = np.where(fl, _COMP[b], b)
                mut = rng.random(tot, dtype=np.float32) < div[i:j][rep]
                nm = int(mut.sum())
                if nm:
                    b[mut] = BASES[(_IDX[b[mut]] + rng.integers(1, 4, size=nm)) % 4]
                for c in range(j - i):
                    a = int(st[i + c])
                    s[a:a + int(lb[c])] = b[cstart[c]:cstart[c] + lb[c]]
                i = j
        is_cg = (s[:-1] == C) & (s[1:] == G)
        pos = np.flatnonzero(is_cg)
        frac = len(pos) / max(1, L)
        keep_p = min(1.0, cpg_frac / frac) if frac > 0 else 1.0
        kp = rng.random(len(pos)) < keep_p
        drop = pos[~kp]
        s[drop + 1] = np.where(rng.random(len(drop)) < 0.5, A, T).astype(np.uint8)
        kept = pos[kp]
        mk = kept[rng.random(len(kept)) < meth_p]
        return s, mk.astype(np.int64), kept.astype(np.int64), copies

    with cf.ThreadPoolExecutor(_threads(threads)) as ex:
        res = list(ex.map(one, range(nchr)))
    if names is None:
        names = ["chr%d" % (i + 1) for i in range(nchr)]
    return LargeGenome(list(names), [r[0] for r in res], [r[1] for r in res], [r[2] for r in res],
                       np.concatenate([r[3] for r in res]) if res else np.zeros((0, 3), np.int64))


def _convert_fragments(genome: LargeGenome, chrom, start, fwd, W, cell_p=None, cell_key=0):
    """Bisulfite-converted fragments of W bases: rows for forward reads are the
    converted forward strand at [start, start + W); rows for reverse reads are
    the reverse complement of the forward-coordinate image of the converted
    reverse strand.  Methylation of a CpG: the genome's state, or, when cell_p
    is given, a per-(cell, site) draw with probability cell_p (a hash of the
    cell key and the site, the same for every read of the cell)."""
    n = len(chrom)
    out = np.empty((n, W), np.uint8)
    cols = np.arange(W, dtype=np.int64)
    for ci in np.unique(chrom):
        sel = np.flatnonzero(chrom == ci)
        s = genome.seqs[ci]
        idx = start[sel, None] + cols[None, :]
        frag = s[idx]
        if cell_p is None:
            mp = genome.meth_pos[ci]
        else:
            cp = genome.cpg_pos[ci]
            h = (cp.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) ^ np.uint64(cell_key * 0xBF58476D1CE4E5B9 & 0xFFFFFFFFFFFFFFFF)
            h ^= h >> np.uint64(31)
            h *= np.uint64(0x94D049BB133111EB)
            h ^= h >> np.uint64(29)
            mp = cp[(h >> np.uint64(11)).astype(np.float64) / float(1 << 53) < cell_p]
        # methylated C positions -> their C (pos) and G (pos + 1) are protected
        j = np.searchsorted(mp, idx[:, 0])
        prot = np.zeros(idx.shape, bool)
        # each fragment holds at most W / 2 CpGs: walk the sorted list in step
        for step in range(W):
            jj = j + step
            inb = jj < len(mp)
            p = np.where(inb, mp[np.minimum(jj, len(mp) - 1)], -1) - idx[:, 0]
            live = inb & (p >= 0) & (p < W)
            if not live.any():
                break
            r = np.flatnonzero(live)
            prot[r, p[r]] = True
            q = p[r] + 1
            ok = q < W
            prot[r[ok], q[ok]] = True
        f = fwd[sel]
        ff = frag[f]
        pf = prot[f]
        ff[(ff == C) & ~pf] = T
        fr = frag[~f]
        pr = prot[~f]
        fr[(fr == G) & ~pr] = A
        out[sel[f]] = ff
        out[sel[~f]] = _COMP[fr[:, ::-1]]
    return out


def make_reads_large(genome: LargeGenome, n_reads, seed, read_len=100, sub_rate=0.01, indel_rate=0.001,
                     length_sampler=None, error_sampler=None, repeat_read_frac=0.0, batch=250_000, threads=0,
                     cell_p=None, cell_key=0) -> ReadSet:
    """Single-end bisulfite reads as make_reads (uniform starts, 50/50 strand,
    conversion, substitutions and 1-bp indels at indel_rate / sub_rate times
    each read's substitution rate, optional repeat-copy starts), batches drawn
    from their own spawned streams on a thread pool."""
    import concurrent.futures as cf
    ss = np.random.SeedSequence(seed)
    top, *kids = ss.spawn(1 + (n_reads + batch - 1) // batch)
    rng = np.random.default_rng(top)
    nchr = len(genome.seqs)
    clen = np.array([len(s) for s in genome.seqs], dtype=np.int64)
    pad = 8
    lens = (np.full(n_reads, read_len, dtype=np.int32) if length_sampler is None
            else np.asarray(length_sampler(rng, n_reads), dtype=np.int32))
    maxL = int(lens.max()) if n_reads else read_len
    W = maxL + pad
    chrom = rng.choice(nchr, size=n_reads, p=clen / clen.sum())
    start = (rng.random(n_reads) * (clen[chrom] - W)).astype(np.int64)
    if repeat_read_frac > 0 and len(genome.repeat_copies):
        rr = rng.random(n_reads) < repeat_read_frac
        cps = genome.repeat_copies
        pick = cps[rng.integers(0, len(cps), size=int(rr.sum()))]
        off = (rng.random(len(pick)) * np.maximum(1, pick[:, 2] - maxL)).astype(np.int64)
        chrom[rr] = pick[:, 0]
        start[rr] = np.minimum(pick[:, 1] + off, clen[pick[:, 0]] - W)
    fwd = rng.random(n_reads) < 0.5
    rates = (np.full(n_reads, sub_rate) if error_sampler is None
             else np.asarray(error_sampler(rng, n_reads), dtype=np.float64))
    irates = rates * (indel_rate / sub_rate if sub_rate > 0 else 0.0)
    out = np.zeros((n_reads, maxL), dtype=np.uint8)

    def one(bi):
        b0 = bi * batch
        b1 = min(n_reads, b0 + batch)
        nb = b1 - b0
        r = np.random.default_rng(kids[bi])
        frag = _convert_fragments(genome, chrom[b0:b1], start[b0:b1], fwd[b0:b1], W, cell_p, cell_key)
        sub = r.random((nb, W), dtype=np.float32) < rates[b0:b1, None]
        ns = int(sub.sum())
        if ns:
            frag[sub] = BASES[(_IDX[frag[sub]] + r.integers(1, 4, size=ns)) % 4]
        nev = r.binomial(maxL, np.minimum(1.0, irates[b0:b1]))
        j = np.arange(W)[None, :]
        for _ in range(int(nev.max()) if nb else 0):
            rows = np.flatnonzero(nev > 0)
            nev[rows] -= 1
            p = r.integers(0, maxL, size=len(rows))
            ins = r.random(len(rows)) < 0.5
            src = np.where(j < p[:, None], j, np.where(ins[:, None], j - 1, j + 1))
            src = np.clip(src, 0, W - 1)
            new = np.take_along_axis(frag[rows], src, axis=1)
            new[ins, p[ins]] = BASES[r.integers(0, 4, size=int(ins.sum()))]
            frag[rows] = new
        blk = frag[:, :maxL]
        blk[np.arange(maxL)[None, :] >= lens[b0:b1, None]] = 0
        out[b0:b1] = blk

    with cf.ThreadPoolExecutor(_threads(threads)) as ex:
        list(ex.map(one, range(len(kids))))
    return ReadSet(out, lens, chrom.astype(np.int32), start, fwd)


def _errors_inplace(r, frag, rates, irates, maxL):
    """Substitutions at each row's rate, then 1-bp indels (one event per pass)
    inside the first maxL columns; frag is (n, W) with W > maxL."""
    nb, W = frag.shape
    sub = r.random((nb, W), dtype=np.float32) < rates[:, None]
    ns = int(sub.sum())
    if ns:
        frag[sub] = BASES[(_IDX[frag[sub]] + r.integers(1, 4, size=ns)) % 4]
    nev = r.binomial(maxL, np.minimum(1.0, irates))
    j = np.arange(W)[None, :]
    for _ in range(int(nev.max()) if nb else 0):
        rows = np.flatnonzero(nev > 0)
        nev[rows] -= 1
        p = r.integers(0, maxL, size=len(rows))
        ins = r.random(len(rows)) < 0.5
        src = np.where(j < p[:, None], j, np.where(ins[:, None], j - 1, j + 1))
        src = np.clip(src, 0, W - 1)
        new = np.take_along_axis(frag[rows], src, axis=1)
        new[ins, p[ins]] = BASES[r.integers(0, 4, size=int(ins.sum()))]
        frag[rows] = new


def make_pairs_large(genome: LargeGenome, n_pairs, seed, read_len=100, inner=(20, 400), sub_rate=0.01,
                     indel_rate=0.001, batch=250_000, threads=0):
    """Paired-end bisulfite reads as make_pairs: a fragment of read_len + inner +
    read_len bases (inner uniform in the closed range) from a random strand;
    mate 1 is its first read_len bases, mate 2 the reverse complement of its
    last read_len bases; substitutions and 1-bp indels per mate."""
    import concurrent.futures as cf
    ss = np.random.SeedSequence(seed)
    top, *kids = ss.spawn(1 + (n_pairs + batch - 1) // batch)
    rng = np.random.default_rng(top)
    nchr = len(genome.seqs)
    clen = np.array([len(s) for s in genome.seqs], dtype=np.int64)
    flen = read_len + rng.integers(inner[0], inner[1] + 1, size=n_pairs) + read_len
    W = 2 * read_len + inner[1] + 8
    chrom = rng.choice(nchr, size=n_pairs, p=clen / clen.sum())
    start = (rng.random(n_pairs) * (clen[chrom] - W)).astype(np.int64)
    fwd = rng.random(n_pairs) < 0.5
    m1 = np.zeros((n_pairs, read_len), np.uint8)
    m2 = np.zeros((n_pairs, read_len), np.uint8)
    cols = np.arange(read_len)

    def one(bi):
        b0 = bi * batch
        b1 = min(n_pairs, b0 + batch)
        r = np.random.default_rng(kids[bi])
        frag = _convert_fragments(genome, chrom[b0:b1], start[b0:b1], fwd[b0:b1], W)
        fl = flen[b0:b1]
        a = frag[:, :read_len + 8].copy()
        b = _COMP[np.take_along_axis(frag, (fl - 1)[:, None] - np.arange(read_len + 8)[None, :] % W, axis=1)]
        rates = np.full(b1 - b0, sub_rate)
        irates = rates * (indel_rate / sub_rate if sub_rate > 0 else 0.0)
        _errors_inplace(r, a, rates, irates, read_len)
        _errors_inplace(r, b, rates, irates, read_len)
        m1[b0:b1] = a[:, :read_len]
        m2[b0:b1] = b[:, :read_len]

    with cf.ThreadPoolExecutor(_threads(threads)) as ex:
        list(ex.map(one, range(len(kids))))
    lens = np.full(n_pairs, read_len, np.int32)
    return (ReadSet(m1, lens, chrom.astype(np.int32), start, fwd),
            ReadSet(m2, lens.copy(), chrom.astype(np.int32), start, ~fwd))
