"""Host-side mirror of FAME's ReadQueue (ReadQueue.h:58-131) over the C ABI.

The names, argument meaning and loop structure follow the reference so that
tests read like its own: parse_chunk (parseChunk, ReadQueue.cpp:218-296),
match_reads (matchReads, 404-933, on the GPU), decide_strand (376-400),
print_methylation_levels (1860-1893) and query_routine (main.cpp:363-399).
"""
from __future__ import annotations

import numpy as np

from ._lib import CHUNKSIZE, FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, HostIndex


class _FastqSource:
    """parseChunk's reading through the native reader (fame_fastq_*): four
    lines per record, sequence = line 2."""

    def __init__(self, path: str, is_gz: bool = False, chunk: int = CHUNKSIZE):
        from ._lib import FastqReader
        self.r = FastqReader(path, is_gz, max_reads=chunk)

    def take(self, n):
        assert n <= self.r.max_reads
        seq, offs = self.r.read()
        return seq.copy(), offs.copy()


class _ListSource:
    def __init__(self, seqs):
        self.seqs = seqs
        self.i = 0

    def take(self, n):
        out = self.seqs[self.i:self.i + n]
        self.i += len(out)
        offs = np.zeros(len(out) + 1, dtype=np.uint64)
        np.cumsum([len(x) for x in out], out=offs[1:])
        return np.frombuffer(b"".join(out), dtype=np.uint8), offs


class ReadQueue:
    def __init__(self, reads, index: HostIndex, gpu: GpuMatcher, is_gz: bool = False, both_strands: bool = False,
                 chunk_size: int = CHUNKSIZE):
        if isinstance(reads, str):
            self.src = _FastqSource(reads, is_gz, chunk_size)
        else:
            self.src = _ListSource(list(reads))
        self.index = index
        self.gpu = gpu
        self.chunk_size = chunk_size
        self.both_strands_flag = both_strands
        self.r1_fwd_matches = 0
        self.r1_rev_matches = 0
        self.match_r1_fwd = True
        self.buffer = (np.zeros(0, np.uint8), np.zeros(1, np.uint64))   # packed sequences, offsets
        self.mats = np.zeros(0, np.uint64)
        self.invalid = np.zeros(0, np.uint8)

    def parse_chunk(self):
        """Returns (procReads, more): more is True iff a full chunk was read."""
        self.buffer = self.src.take(self.chunk_size)
        n = len(self.buffer[1]) - 1
        return n, n >= self.chunk_size

    def match_reads(self, proc_reads: int, get_stranded: bool):
        """Match the first proc_reads reads of the buffer; returns this call's Counters."""
        seq, offs = self.buffer
        offs = offs[:proc_reads + 1]
        flags = (FAME_GET_STRANDED if get_stranded else 0) | (FAME_BOTH_STRANDS if self.both_strands_flag else 0) | \
            (FAME_MATCH_R1_FWD if self.match_r1_fwd else 0)
        mats, inval, cnt = self.gpu.match_reads(seq[: int(offs[-1])], offs, flags)
        self.mats, self.invalid = mats, inval
        self.r1_fwd_matches += cnt.r1_fwd
        self.r1_rev_matches += cnt.r1_rev
        return cnt

    def decide_strand(self):
        self.match_r1_fwd = self.r1_fwd_matches > self.r1_rev_matches

    def methylation_levels(self) -> np.ndarray:
        return self.gpu.tallies(reset=False)

    def print_methylation_levels(self, basename: str):
        """<basename>_cpg.tsv: chrom, C position, methFwd, unmethFwd, methRev, unmethRev."""
        write_cpg_report(basename + "_cpg.tsv", self.index, self.gpu.tallies(reset=False))

    def query_routine(self):
        """main.cpp:363-399; returns the summed counters."""
        tot = dict(succ=0, nonunique=0, unsucc=0)

        def add(c):
            tot["succ"] += c.succ
            tot["nonunique"] += c.nonunique
            tot["unsucc"] += c.unsucc

        if not self.both_strands_flag:
            n, _ = self.parse_chunk()
            add(self.match_reads(n, True))
            self.decide_strand()
        while True:
            n, more = self.parse_chunk()
            if not more:
                break
            add(self.match_reads(n, False))
        add(self.match_reads(n, False))
        return tot


class PairedReadQueue:
    """Paired-end chunk loop: the two-file ReadQueue with matchPairedReads
    (ReadQueue.cpp:940-1658) on the GPU and queryRoutinePaired
    (main.cpp:400-441).  maxpdist is the MAXPDIST of the reference build
    (CONST.h:42)."""

    def __init__(self, reads1, reads2, index: HostIndex, gpu: GpuMatcher, maxpdist: int, is_gz: bool = False,
                 both_strands: bool = False, chunk_size: int = CHUNKSIZE):
        self.src = [(_FastqSource(r, is_gz, chunk_size) if isinstance(r, str) else _ListSource(list(r)))
                    for r in (reads1, reads2)]
        self.index = index
        self.gpu = gpu
        self.maxpdist = maxpdist
        self.chunk_size = chunk_size
        self.both_strands_flag = both_strands
        self.r1_fwd_matches = 0
        self.r1_rev_matches = 0
        self.match_r1_fwd = True
        self.buffer = ((np.zeros(0, np.uint8), np.zeros(1, np.uint64)),) * 2
        self.mats = (np.zeros(0, np.uint64), np.zeros(0, np.uint64))
        self.invalid = (np.zeros(0, np.uint8), np.zeros(0, np.uint8))

    def parse_chunk(self):
        """Returns (procReads, more): the pairs read, more iff a full chunk was read."""
        b1 = self.src[0].take(self.chunk_size)
        b2 = self.src[1].take(self.chunk_size)
        n = len(b1[1]) - 1
        if len(b2[1]) - 1 != n:
            raise ValueError("mate files hold different numbers of reads")
        self.buffer = (b1, b2)
        return n, n >= self.chunk_size

    def match_paired_reads(self, proc_reads: int, get_stranded: bool):
        """Match pairs buffer[:proc_reads]; returns this call's PairCounters."""
        packed = []
        for seq, offs in self.buffer:
            offs = offs[:proc_reads + 1]
            packed.append((seq[: int(offs[-1])], offs))
        flags = (FAME_GET_STRANDED if get_stranded else 0) | (FAME_BOTH_STRANDS if self.both_strands_flag else 0) | \
            (FAME_MATCH_R1_FWD if self.match_r1_fwd else 0)
        m1, m2, i1, i2, cnt = self.gpu.match_pairs(packed[0][0], packed[0][1], packed[1][0], packed[1][1], flags,
                                                   self.maxpdist)
        self.mats, self.invalid = (m1, m2), (i1, i2)
        self.r1_fwd_matches += cnt.r1_fwd
        self.r1_rev_matches += cnt.r1_rev
        return cnt

    def decide_strand(self):
        self.match_r1_fwd = self.r1_fwd_matches > self.r1_rev_matches

    def print_methylation_levels(self, basename: str):
        write_cpg_report(basename + "_cpg.tsv", self.index, self.gpu.tallies(reset=False))

    def query_routine_paired(self):
        """main.cpp:400-441; returns the summed counters."""
        keys = ("succ", "nonunique", "unsucc", "paired", "too_short")
        tot = dict.fromkeys(keys, 0)

        def add(c):
            for k in keys:
                tot[k] += getattr(c, k)

        if not self.both_strands_flag:
            n, _ = self.parse_chunk()
            add(self.match_paired_reads(n, True))
            self.decide_strand()
        while True:
            n, more = self.parse_chunk()
            if not more:
                break
            add(self.match_paired_reads(n, False))
        add(self.match_paired_reads(n, False))
        return tot


def write_cpg_report(path: str, index: HostIndex, meth: np.ndarray, n_threads: int = 0):
    """printMethylationLevels (ReadQueue.cpp:1860-1893), by the native writer."""
    import ctypes as C
    from ._lib import _check, _ptr, lib
    m = np.ascontiguousarray(meth, dtype=np.uint16)
    _check(lib().fame_report_cpg(C.byref(index.view), _ptr(m), path.encode(), n_threads))


class SingleCellQueue:
    """Single-cell batches (matchSCBatch, ReadQueue.cpp:1660-1748, and
    printSCMethylationLevels, 1894-1921; queryRoutineSC, main.cpp:443-468).

    Per cell: the strand votes restart at zero, the cell's reads run through
    the chunk loop (first chunk with getStranded unless both_strands), then the
    cell's four count rows are written and the counters zeroed.  As in the
    reference, the final bulk report after all cells is therefore all zeros,
    and the fourth row is labelled "unmethFwd" (ReadQueue.cpp:1915)."""

    def __init__(self, out_path: str, index: HostIndex, gpu: GpuMatcher, both_strands: bool = False,
                 chunk_size: int = CHUNKSIZE):
        import ctypes as C
        from ._lib import _check, lib
        self.index = index
        self.gpu = gpu
        self.both = both_strands
        self.chunk_size = chunk_size
        self.path = out_path
        _check(lib().fame_report_sc_header(C.byref(index.view), out_path.encode()))

    def match_sc_batch(self, reads, sc_id: str):
        rq = ReadQueue(reads, self.index, self.gpu, both_strands=self.both, chunk_size=self.chunk_size)
        tot = rq.query_routine()
        self.print_sc_methylation_levels(sc_id)
        return tot

    def print_sc_methylation_levels(self, sc_id: str):
        import ctypes as C
        from ._lib import _check, _ptr, lib
        meth = np.ascontiguousarray(self.gpu.tallies(reset=True), dtype=np.uint16)
        _check(lib().fame_report_sc_rows(C.byref(self.index.view), sc_id.encode(), _ptr(meth), self.path.encode(), 0))

    def close(self):
        pass


def read_sc_meta(path: str):
    """queryRoutineSC's meta file: '<id> <fastq path>' per line, split on spaces (main.cpp:454-458)."""
    out = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            p = line.find(" ")
            sc_id = line[:p] if p >= 0 else line
            rest = line[p + 1:] if p >= 0 else ""
            q = rest.find(" ")
            out.append((sc_id, rest[:q] if q >= 0 else rest))
    return out
