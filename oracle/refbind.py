"""Test infrastructure: ctypes binding of oracle/_ref/libfame_ref.so (the
reference FAME sources compiled by oracle/build_ref.sh).  Used only by the
golden-fixture script, the oracle tests and bench.py's CPU baseline."""
from __future__ import annotations

import ctypes as C
import os
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libfame_ref.so")
# the constant sets oracle/build_ref.sh compiles: (READLEN, MAXPDIST) -> library
VARIANTS = {(100, 550): LIB_PATH,
            (150, 550): os.path.join(HERE, "_ref", "libfame_ref_rl150.so"),
            (100, 400): os.path.join(HERE, "_ref", "libfame_ref_pd400.so")}

_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def variant_path(readlen: int = 100, maxpdist: int = 550) -> str:
    """Library of the reference compiled with these CONST.h values (KeyError if none is built)."""
    return VARIANTS[(int(readlen), int(maxpdist))]


def available(readlen: int = 100, maxpdist: int = 550) -> bool:
    p = VARIANTS.get((int(readlen), int(maxpdist)))
    return p is not None and os.path.exists(p)


class RefLib:
    def __init__(self, path: str = LIB_PATH):
        self.lib = C.CDLL(path)
        L = self.lib
        L.fame_ref_build.restype = _P
        L.fame_ref_build.argtypes = [C.c_char_p, C.c_int]
        L.fame_ref_load.restype = _P
        L.fame_ref_load.argtypes = [C.c_char_p]
        L.fame_ref_from_arrays.restype = _P
        L.fame_ref_free.argtypes = [_P]
        L.fame_ref_sizes.argtypes = [_P, _P]
        L.fame_ref_match_se.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_int, _P, _P, _P, _P, _P]
        L.fame_ref_seed_order.argtypes = [_P, C.c_char_p, C.c_uint32, C.c_uint32, _P, _P, _P]
        L.fame_ref_lev.argtypes = [C.c_int, C.c_char_p, C.c_uint32, C.c_char_p, C.c_int, C.c_int, _P, C.c_uint32, _P]
        L.fame_ref_shiftand.argtypes = [C.c_char_p, C.c_uint32, C.c_char_p, C.c_uint32, C.c_int, _P, _P, C.c_uint32]
        self.corenum = L.fame_ref_corenum()
        self.readlen = L.fame_ref_readlen()
        self.maxpdist_value = L.fame_ref_maxpdist()

    def maxpdist(self) -> int:
        return int(self.maxpdist_value)

    # --- index -------------------------------------------------------------
    def build(self, fasta: str, noloss: bool = False):
        return RefIndex(self, self.lib.fame_ref_build(fasta.encode(), int(noloss)))

    def from_arrays(self, ix) -> "RefIndex":
        """ix: an object with the loaded-index arrays (see fame_gb300.index.HostIndex)."""
        nch = len(ix.chrom_seqs)
        seqs = [np.ascontiguousarray(s) for s in ix.chrom_seqs]
        seq_ptrs = (C.c_void_p * nch)(*[s.ctypes.data for s in seqs])
        lens = np.array([len(s) for s in seqs], dtype=np.uint64)
        names = (C.c_char_p * nch)(*[n.encode() for n in ix.chrom_names])
        L = self.lib
        L.fame_ref_from_arrays.argtypes = [C.c_uint32, _P, _P, _P, C.c_uint64, _P, _P, C.c_uint64, _P, _P, _P,
                                           C.c_uint64, _P, _P, _P, C.c_uint64, _P, _P, _P, _P, C.c_uint64, _P]
        h = L.fame_ref_from_arrays(
            nch, C.cast(seq_ptrs, C.c_void_p), _ptr(lens), C.cast(names, C.c_void_p),
            len(ix.cpg_pos), _ptr(ix.cpg_chrom), _ptr(ix.cpg_pos),
            len(ix.cpgs_pos), _ptr(ix.cpgs_chrom), _ptr(ix.cpgs_pos),
            _ptr(ix.tab_index64()),
            len(ix.kmer_meta), _ptr(ix.kmer_meta), _ptr(ix.kmer_tmask), _ptr(ix.strand),
            len(ix.win_start), _ptr(ix.win_start), _ptr(ix.win_chrom), _ptr(ix.win_sind), _ptr(ix.win_eind),
            len(ix.filtered), _ptr(ix.filtered))
        return RefIndex(self, h)

    def lev(self, band, row: bytes, col: bytes, col_end: int, rev: int, comp: int):
        """Reference LevenshtDP with colPat = col[col_end]; returns (dist, trace list)."""
        buf = C.create_string_buffer(col, len(col))
        cptr = C.cast(C.addressof(buf) + col_end, C.c_char_p)
        tr = np.zeros(4096, dtype=np.uint8)
        d = np.zeros(1, dtype=np.uint32)
        n = self.lib.fame_ref_lev(band, row, len(row), cptr, rev, comp, _ptr(tr), 4096, _ptr(d))
        return int(d[0]), tr[:n].tolist()

    def shiftand(self, pat: bytes, text: bytes, rev: int):
        offs = np.zeros(4096, dtype=np.uint64)
        errs = np.zeros(4096, dtype=np.uint8)
        n = self.lib.fame_ref_shiftand(pat, len(pat), text, len(text), rev, _ptr(offs), _ptr(errs), 4096)
        return offs[:n].tolist(), errs[:n].tolist()


class RefIndex:
    def __init__(self, lib: RefLib, handle):
        self.L = lib
        self.h = handle

    def close(self):
        if self.h:
            self.L.lib.fame_ref_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dump(self) -> dict:
        sz = np.zeros(7, dtype=np.uint64)
        self.L.lib.fame_ref_sizes(self.h, _ptr(sz))
        ncpg, ncpgs, nch, nb, nk, nw, nf = (int(x) for x in sz)
        d = dict(cpg_chrom=np.zeros(ncpg, np.uint8), cpg_pos=np.zeros(ncpg, np.uint32),
                 cpgs_chrom=np.zeros(ncpgs, np.uint8), cpgs_pos=np.zeros(ncpgs, np.uint32),
                 bucket_key=np.zeros(nb, np.uint32), bucket_start=np.zeros(nb, np.uint64),
                 bucket_len=np.zeros(nb, np.uint32), kmer_meta=np.zeros(nk, np.uint32),
                 kmer_tmask=np.zeros(nk, np.uint32), strand=np.zeros(nk, np.uint8),
                 win_start=np.zeros(nw, np.uint32), win_chrom=np.zeros(nw, np.uint8),
                 win_sind=np.zeros(nw, np.uint32), win_eind=np.zeros(nw, np.uint32),
                 filtered=np.zeros(nf, np.uint64))
        L = self.L.lib
        L.fame_ref_dump.argtypes = [_P] * 16
        L.fame_ref_dump(self.h, *[_ptr(d[k]) for k in (
            "cpg_chrom", "cpg_pos", "cpgs_chrom", "cpgs_pos", "bucket_key", "bucket_start", "bucket_len",
            "kmer_meta", "kmer_tmask", "strand", "win_start", "win_chrom", "win_sind", "win_eind", "filtered")])
        return d

    def match_se(self, seq_bytes: bytes, offs: np.ndarray, chunk: int = 0, both_strands: bool = False,
                 n_cpg: int | None = None):
        n = len(offs) - 1
        if n_cpg is None:
            sz = np.zeros(7, dtype=np.uint64)
            self.L.lib.fame_ref_sizes(self.h, _ptr(sz))
            n_cpg = int(sz[0])
        mats = np.zeros(n, np.uint64)
        inval = np.zeros(n, np.uint8)
        meth = np.zeros(4 * n_cpg, np.uint16)
        cnt = np.zeros(6, np.uint64)
        secs = np.zeros(1, np.float64)
        buf = np.frombuffer(seq_bytes, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        self.L.lib.fame_ref_match_se(self.h, _ptr(buf), _ptr(offs), n, chunk, int(both_strands),
                                     _ptr(mats), _ptr(inval), _ptr(meth), _ptr(cnt), _ptr(secs))
        return dict(mat=mats, invalid=inval, meth=meth.reshape(-1, 4), counters=cnt, seconds=float(secs[0]))

    def _n_cpg(self) -> int:
        sz = np.zeros(7, dtype=np.uint64)
        self.L.lib.fame_ref_sizes(self.h, _ptr(sz))
        return int(sz[0])

    def time_se(self, seq_bytes: bytes, offs: np.ndarray, both_strands: bool = False, match_r1_fwd: bool = True,
                outputs: bool = False):
        """Seconds spent in matchReads for already-stranded chunks, and [succ,
        nonunique, unsucc]; with outputs, also a dict of the run's per-read mat
        and invalid and its methLevels (read after the timed calls)."""
        import ctypes as C
        f = self.L.lib.fame_ref_time_se
        f.argtypes = [_P, _P, _P, C.c_uint32, C.c_int, C.c_int, _P, _P, _P, _P, _P]
        n = len(offs) - 1
        cnt = np.zeros(3, np.uint64)
        secs = np.zeros(1, np.float64)
        buf = np.frombuffer(seq_bytes, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        out = None
        if outputs:
            out = dict(mat=np.zeros(n, np.uint64), invalid=np.zeros(n, np.uint8),
                       meth=np.zeros(4 * self._n_cpg(), np.uint16))
        f(self.h, _ptr(buf), _ptr(offs), n, int(both_strands), int(match_r1_fwd), _ptr(cnt), _ptr(secs),
          *((_ptr(out["mat"]), _ptr(out["invalid"]), _ptr(out["meth"])) if out else (None, None, None)))
        if out:
            out["meth"] = out["meth"].reshape(-1, 4)
            return float(secs[0]), cnt, out
        return float(secs[0]), cnt

    def time_pe(self, s1: bytes, o1, s2: bytes, o2, both_strands: bool = False, match_r1_fwd: bool = True,
                outputs: bool = False):
        """Seconds spent in matchPairedReads for already-stranded chunks, and
        [succ, nonunique, unsucc, succPaired, tooShort]; with outputs, also a
        dict of mat1, mat2, inv1, inv2 and methLevels of the run."""
        import ctypes as C
        f = self.L.lib.fame_ref_time_pe
        f.argtypes = [_P, _P, _P, _P, _P, C.c_uint32, C.c_int, C.c_int, _P, _P, _P, _P, _P]
        n = len(o1) - 1
        cnt = np.zeros(5, np.uint64)
        secs = np.zeros(1, np.float64)
        b1 = np.frombuffer(s1, np.uint8)
        b2 = np.frombuffer(s2, np.uint8)
        o1 = np.ascontiguousarray(o1, np.uint64)
        o2 = np.ascontiguousarray(o2, np.uint64)
        mats = inv = meth = None
        if outputs:
            mats = np.zeros(2 * n, np.uint64)
            inv = np.zeros(2 * n, np.uint8)
            meth = np.zeros(4 * self._n_cpg(), np.uint16)
        f(self.h, _ptr(b1), _ptr(o1), _ptr(b2), _ptr(o2), n, int(both_strands), int(match_r1_fwd), _ptr(cnt),
          _ptr(secs), _ptr(mats), _ptr(inv), _ptr(meth))
        if outputs:
            return float(secs[0]), cnt, dict(mat1=mats[:n], mat2=mats[n:], inv1=inv[:n], inv2=inv[n:],
                                             meth=meth.reshape(-1, 4))
        return float(secs[0]), cnt

    def match_pe(self, s1: bytes, o1, s2: bytes, o2, chunk: int = 0, both_strands: bool = False):
        import ctypes as C
        f = self.L.lib.fame_ref_match_pe
        f.argtypes = [_P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_int, _P, _P, _P, _P, _P, _P, _P]
        sz = np.zeros(7, dtype=np.uint64)
        self.L.lib.fame_ref_sizes(self.h, _ptr(sz))
        n = len(o1) - 1
        m1 = np.zeros(n, np.uint64)
        m2 = np.zeros(n, np.uint64)
        i1 = np.zeros(n, np.uint8)
        i2 = np.zeros(n, np.uint8)
        meth = np.zeros(4 * int(sz[0]), np.uint16)
        cnt = np.zeros(8, np.uint64)
        secs = np.zeros(1, np.float64)
        b1 = np.frombuffer(s1, np.uint8)
        b2 = np.frombuffer(s2, np.uint8)
        o1 = np.ascontiguousarray(o1, np.uint64)
        o2 = np.ascontiguousarray(o2, np.uint64)
        f(self.h, _ptr(b1), _ptr(o1), _ptr(b2), _ptr(o2), n, chunk, int(both_strands), _ptr(m1), _ptr(m2), _ptr(i1),
          _ptr(i2), _ptr(meth), _ptr(cnt), _ptr(secs))
        return dict(mat1=m1, mat2=m2, inv1=i1, inv2=i2, meth=meth.reshape(-1, 4), counters=cnt, seconds=float(secs[0]))

    def print_cpg(self, meth, basename: str) -> str:
        """The reference's printMethylationLevels of these tallies; returns the file path."""
        f = self.L.lib.fame_ref_print_cpg
        f.argtypes = [_P, _P, C.c_char_p]
        m = np.ascontiguousarray(meth, np.uint16)
        f(self.h, _ptr(m), basename.encode())
        return basename + "_cpg.tsv"

    def print_sc(self, path: str, cells):
        """The reference's single-cell matrix for [(cell id, tallies)]."""
        f = self.L.lib.fame_ref_print_sc
        f.argtypes = [_P, C.c_char_p, C.c_uint32, _P, _P]
        ids = (C.c_char_p * len(cells))(*[c.encode() for c, _ in cells])
        m = np.ascontiguousarray(np.stack([np.asarray(x, np.uint16) for _, x in cells]), np.uint16)
        f(self.h, path.encode(), len(cells), C.cast(ids, C.c_void_p), _ptr(m))

    def seed_order(self, seq: bytes, cap: int = 1 << 20):
        keys = np.zeros(cap, np.uint32)
        cnts = np.zeros(cap, np.uint32)
        nout = np.zeros(4, np.uint64)
        rc = self.L.lib.fame_ref_seed_order(self.h, seq, len(seq), cap, _ptr(keys), _ptr(cnts), _ptr(nout))
        if rc != 0:
            raise RuntimeError("seed order overflow")
        nf, nr = int(nout[0]), int(nout[1])
        return (list(zip(keys[:nf].tolist(), cnts[:nf].tolist())),
                list(zip(keys[nf:nf + nr].tolist(), cnts[nf:nf + nr].tolist())),
                int(nout[2]), int(nout[3]))
