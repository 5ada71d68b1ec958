"""Test infrastructure: ctypes binding of the C restatement (oracle/fame_oracle.c).

Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
the parity checker; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_P = C.c_void_p


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class _Index(C.Structure):
    _fields_ = [("readlen", C.c_uint32), ("n_chrom", C.c_uint32), ("chrom_seq", _P), ("chrom_len", _P),
                ("n_cpg", C.c_uint64), ("cpg_chrom", _P), ("cpg_pos", _P),
                ("n_bucket", C.c_uint64), ("bucket_key", _P), ("bucket_start", _P), ("bucket_len", _P),
                ("n_kmer", C.c_uint64), ("kmer_meta", _P), ("strand", _P),
                ("n_win", C.c_uint64), ("win_start", _P), ("win_chrom", _P), ("win_sind", _P), ("win_eind", _P)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_build.restype = _P
        L.orc_build.argtypes = [C.c_uint32, C.c_uint32, _P, _P, C.c_int]
        L.orc_built_sizes.argtypes = [_P, _P]
        L.orc_built_copy.argtypes = [_P] * 17
        L.orc_built_free.argtypes = [_P]
        L.orc_match_se.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_int, _P, _P, _P, _P]
        L.orc_seed_order.argtypes = [_P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]
        L.orc_lev.argtypes = [C.c_int, _P, C.c_uint32, _P, C.c_int64, C.c_int64, C.c_int, C.c_int, _P, C.c_uint32, _P]
        L.orc_shiftand.argtypes = [_P, C.c_uint32, _P, C.c_uint32, C.c_int, _P, _P, C.c_uint32]
        L.orc_match_chunk.argtypes = [_P, _P, _P, C.c_uint32, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P]
        L.orc_match_pe.argtypes = [_P, _P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_int, _P, _P, _P, _P, _P, _P]
        L.orc_sort_desc.argtypes = [_P, _P, C.c_uint32, _P]
        _lib = L
    return _lib


class _PeExtra(C.Structure):
    _fields_ = [("kmer_tmask", _P), ("n_filtered", C.c_uint64), ("filtered", _P), ("maxpdist", C.c_uint32)]


def sort_desc(keys, counts):
    keys = np.ascontiguousarray(keys, np.uint32)
    counts = np.ascontiguousarray(counts, np.uint8)
    out = np.zeros(len(keys), np.uint32)
    lib().orc_sort_desc(_ptr(keys), _ptr(counts), len(keys), _ptr(out))
    return out


class OracleIndex:
    """Loaded-index tables (sparse bucket form) as numpy arrays + the C view."""

    FIELDS = ("cpg_chrom", "cpg_pos", "cpgs_chrom", "cpgs_pos", "bucket_key", "bucket_start", "bucket_len",
              "kmer_meta", "kmer_tmask", "strand", "win_start", "win_chrom", "win_sind", "win_eind", "filtered")

    def __init__(self, readlen: int, chrom_seqs, tables: dict, chrom_names=None):
        self.readlen = int(readlen)
        self.chrom_seqs = [np.ascontiguousarray(s, dtype=np.uint8) for s in chrom_seqs]
        self.chrom_names = list(chrom_names) if chrom_names else ["chr%d" % (i + 1) for i in range(len(chrom_seqs))]
        self.t = {k: np.ascontiguousarray(tables[k]) for k in self.FIELDS if k in tables}
        self._seq_ptrs = (C.c_void_p * len(self.chrom_seqs))(*[s.ctypes.data for s in self.chrom_seqs])
        self._lens = np.array([len(s) for s in self.chrom_seqs], dtype=np.uint64)
        t = self.t
        self.view = _Index(self.readlen, len(self.chrom_seqs), C.cast(self._seq_ptrs, _P), _ptr(self._lens),
                           len(t["cpg_pos"]), _ptr(t["cpg_chrom"]), _ptr(t["cpg_pos"]),
                           len(t["bucket_key"]), _ptr(t["bucket_key"]), _ptr(t["bucket_start"]), _ptr(t["bucket_len"]),
                           len(t["kmer_meta"]), _ptr(t["kmer_meta"]), _ptr(t["strand"]),
                           len(t["win_start"]), _ptr(t["win_start"]), _ptr(t["win_chrom"]), _ptr(t["win_sind"]),
                           _ptr(t["win_eind"]))

    @property
    def n_cpg(self) -> int:
        return int(len(self.t["cpg_pos"]))

    @classmethod
    def build(cls, chrom_raw, readlen: int = 100, noloss: bool = False, chrom_names=None) -> "OracleIndex":
        """Index build as RefReader_istr + RefGenome ctor (restated in fame_oracle.c)."""
        L = lib()
        raws = [np.ascontiguousarray(s, dtype=np.uint8) for s in chrom_raw]
        ptrs = (C.c_void_p * len(raws))(*[s.ctypes.data for s in raws])
        lens = np.array([len(s) for s in raws], dtype=np.uint64)
        h = L.orc_build(readlen, len(raws), C.cast(ptrs, _P), _ptr(lens), int(noloss))
        sz = np.zeros(6, dtype=np.uint64)
        L.orc_built_sizes(h, _ptr(sz))
        ncpg, ncpgs, nb, nk, nw, nf = (int(x) for x in sz)
        t = dict(cpg_chrom=np.zeros(ncpg, np.uint8), cpg_pos=np.zeros(ncpg, np.uint32),
                 cpgs_chrom=np.zeros(ncpgs, np.uint8), cpgs_pos=np.zeros(ncpgs, np.uint32),
                 bucket_key=np.zeros(nb, np.uint32), bucket_start=np.zeros(nb, np.uint64),
                 bucket_len=np.zeros(nb, np.uint32), kmer_meta=np.zeros(nk, np.uint32),
                 kmer_tmask=np.zeros(nk, np.uint32), strand=np.zeros(nk, np.uint8),
                 win_start=np.zeros(nw, np.uint32), win_chrom=np.zeros(nw, np.uint8),
                 win_sind=np.zeros(nw, np.uint32), win_eind=np.zeros(nw, np.uint32),
                 filtered=np.zeros(nf, np.uint64))
        seqs = [np.zeros(len(s), np.uint8) for s in raws]
        sptrs = (C.c_void_p * len(seqs))(*[s.ctypes.data for s in seqs])
        L.orc_built_copy(h, *[_ptr(t[k]) for k in cls.FIELDS], C.cast(sptrs, _P))
        L.orc_built_free(h)
        return cls(readlen, seqs, t, chrom_names)

    def match_se(self, seq_bytes: bytes, offs, chunk: int = 0, both_strands: bool = False) -> dict:
        n = len(offs) - 1
        mats = np.zeros(n, np.uint64)
        inval = np.zeros(n, np.uint8)
        meth = np.zeros(4 * self.n_cpg, np.uint16)
        cnt = np.zeros(6, np.uint64)
        buf = np.frombuffer(seq_bytes, dtype=np.uint8)
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        lib().orc_match_se(C.byref(self.view), _ptr(buf), _ptr(offs), n, chunk, int(both_strands),
                           _ptr(mats), _ptr(inval), _ptr(meth), _ptr(cnt))
        return dict(mat=mats, invalid=inval, meth=meth.reshape(-1, 4), counters=cnt)

    def match_chunk(self, seq_bytes, offs, get_stranded: bool, both_strands: bool, match_r1_fwd: bool, meth):
        """One matchReads call; meth (uint16, 4 per CpG) accumulates.  Returns mats, invalid, counters[5]."""
        n = len(offs) - 1
        mats = np.zeros(n, np.uint64)
        inval = np.zeros(n, np.uint8)
        cnt = np.zeros(5, np.uint64)
        buf = np.frombuffer(seq_bytes, dtype=np.uint8) if isinstance(seq_bytes, (bytes, bytearray)) else seq_bytes
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        lib().orc_match_chunk(C.byref(self.view), _ptr(buf), _ptr(offs), n, int(get_stranded), int(both_strands),
                              int(match_r1_fwd), _ptr(mats), _ptr(inval), _ptr(meth), _ptr(cnt))
        return mats, inval, cnt

    def match_pe(self, s1: bytes, o1, s2: bytes, o2, chunk: int = 0, both_strands: bool = False,
                 maxpdist: int = 550) -> dict:
        n = len(o1) - 1
        px = _PeExtra(_ptr(self.t["kmer_tmask"]), len(self.t["filtered"]), _ptr(self.t["filtered"]), maxpdist)
        m1 = np.zeros(n, np.uint64)
        m2 = np.zeros(n, np.uint64)
        i1 = np.zeros(n, np.uint8)
        i2 = np.zeros(n, np.uint8)
        meth = np.zeros(4 * self.n_cpg, np.uint16)
        cnt = np.zeros(8, np.uint64)
        b1 = np.frombuffer(s1, np.uint8)
        b2 = np.frombuffer(s2, np.uint8)
        o1 = np.ascontiguousarray(o1, np.uint64)
        o2 = np.ascontiguousarray(o2, np.uint64)
        lib().orc_match_pe(C.byref(self.view), C.byref(px), _ptr(b1), _ptr(o1), _ptr(b2), _ptr(o2), n, chunk,
                           int(both_strands), _ptr(m1), _ptr(m2), _ptr(i1), _ptr(i2), _ptr(meth), _ptr(cnt))
        return dict(mat1=m1, mat2=m2, inv1=i1, inv2=i2, meth=meth.reshape(-1, 4), counters=cnt)

    def seed_order(self, seq: bytes, cap: int = 1 << 20):
        keys = np.zeros(cap, np.uint32)
        cnts = np.zeros(cap, np.uint32)
        nout = np.zeros(4, np.uint64)
        s = np.frombuffer(seq, dtype=np.uint8)
        rc = lib().orc_seed_order(C.byref(self.view), _ptr(s), len(seq), cap, _ptr(keys), _ptr(cnts), _ptr(nout))
        if rc != 0:
            raise RuntimeError("seed order overflow")
        nf, nr = int(nout[0]), int(nout[1])
        return (list(zip(keys[:nf].tolist(), cnts[:nf].tolist())),
                list(zip(keys[nf:nf + nr].tolist(), cnts[nf:nf + nr].tolist())),
                int(nout[2]), int(nout[3]))


def lev(band: int, row: bytes, col: bytes, col_end: int, rev: int, comp: int):
    r = np.frombuffer(row, dtype=np.uint8)
    c = np.frombuffer(col, dtype=np.uint8)
    tr = np.zeros(4096, np.uint8)
    d = np.zeros(1, np.uint32)
    n = lib().orc_lev(band, _ptr(r), len(row), _ptr(c), len(col), col_end, rev, comp, _ptr(tr), 4096, _ptr(d))
    return int(d[0]), tr[:n].tolist()


def shiftand(pat: bytes, text: bytes, rev: int):
    p = np.frombuffer(pat, dtype=np.uint8)
    t = np.frombuffer(text, dtype=np.uint8)
    offs = np.zeros(4096, np.uint64)
    errs = np.zeros(4096, np.uint8)
    n = lib().orc_shiftand(_ptr(p), len(pat), _ptr(t), len(text), rev, _ptr(offs), _ptr(errs), 4096)
    return offs[:n].tolist(), errs[:n].tolist()
