"""ctypes binding of libfame_gpu.so (the C ABI declared in include/fame_gpu.h).

The library is the product; this module only marshals numpy buffers.  It
raises on import-time use when the library has not been built, so no caller
can silently run without the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os
import numpy as np

from . import build as _build

_P = C.c_void_p
HTABSIZE = 1 << 30
CHUNKSIZE = 300000

FAME_GET_STRANDED = 1
FAME_BOTH_STRANDS = 2
FAME_MATCH_R1_FWD = 4
FAME_MAX_READ_LEN = 255

ERRORS = {0: "FAME_OK", -1: "FAME_ERR_ARG", -2: "FAME_ERR_CUDA", -3: "FAME_ERR_NOMEM", -4: "FAME_ERR_INDEX",
          -5: "FAME_ERR_READ", -6: "FAME_ERR_IO", -7: "FAME_ERR_TIMEOUT", -8: "FAME_ERR_BUSY"}


class FameError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class IndexView(C.Structure):
    _fields_ = [("readlen", C.c_uint32), ("n_chrom", C.c_uint32), ("chrom_seq", _P), ("chrom_len", _P),
                ("chrom_name", _P), ("n_cpg", C.c_uint64), ("cpg", _P), ("tab_index", _P), ("tab_index32", _P),
                ("n_kmer", C.c_uint64), ("kmer", _P), ("strand_bits", _P), ("n_win", C.c_uint64), ("win", _P),
                ("n_filtered", C.c_uint64), ("filtered", _P)]


class Counters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("succ", "nonunique", "unsucc", "r1_fwd", "r1_rev", "invalid_len",
                                          "invalid_n", "gather_bytes", "windows_scanned", "dp_reads", "heavy_tasks",
                                          "reruns")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class PairCounters(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("succ", "nonunique", "unsucc", "paired", "too_short", "r1_fwd", "r1_rev",
                                          "dp_reads", "heavy_pairs")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


CPG_DT = np.dtype([("chrom", np.uint8), ("pos", np.uint32)], align=True)                 # 8 bytes
WIN_DT = np.dtype([("start_pos", np.uint32), ("chrom", np.uint8), ("start_ind", np.uint32),
                   ("end_ind", np.uint32)], align=True)                                   # 16 bytes
KMER_DT = np.dtype([("meta", np.uint32), ("tmask", np.uint32)])

EXPORTS = ["fame_index_read", "fame_index_build", "fame_index_view_of", "fame_index_free", "fame_index_cpg_start",
           "fame_gpu_open", "fame_gpu_close", "fame_gpu_last_error", "fame_gpu_match_reads",
           "fame_gpu_match_reads_dev", "fame_gpu_tallies", "fame_gpu_alloc", "fame_gpu_free", "fame_gpu_memcpy",
           "fame_gpu_host_alloc", "fame_gpu_host_free", "fame_gpu_stream", "fame_gpu_set_timing",
           "fame_gpu_stage_times", "fame_gpu_last_launches", "fame_gpu_match_pairs", "fame_gpu_match_pairs_dev", "fame_queue_open",
           "fame_queue_submit", "fame_queue_ready", "fame_queue_collect", "fame_queue_launches", "fame_queue_close",
           "fame_gpu_tally_alloc", "fame_gpu_tally_read", "fame_gpu_tally_free", "fame_gpu_mem_info",
           "fame_report_cpg", "fame_report_sc_header", "fame_report_sc_rows", "fame_fastq_open", "fame_fastq_read",
           "fame_fastq_close", "fame_queue_stage", "fame_queue_submit_staged", "fame_match_fastq",
           "fame_match_fastq_paired", "fame_index_write", "fame_gpu_index_bytes", "fame_queue_wait",
           "fame_gpu_set_seed_tier", "fame_gpu_autotune", "fame_gpu_load_tuning",
           "fame_gpu_seed_tier_counts", "fame_gpu_map_order_probe", "fame_gpu_pair_stage_times",
           "fame_gpu_open_layout", "fame_gpu_rec_layout", "fame_index_build_gpu", "fame_index_filtered_order",
           "fame_fastq_open_dev", "fame_fastq_gpu_inflate", "fame_host_page_node", "fame_gpu_host_node"]

_lib = None


def lib(build_if_missing: bool = True):
    """Load libfame_gpu.so (building it first when allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise ImportError("libfame_gpu.so is not built (run fame_gb300.build.build())")
        _build.build()
    L = C.CDLL(_build.LIB)
    L.fame_index_read.argtypes = [C.c_char_p, _P]
    L.fame_index_write.argtypes = [_P, C.c_char_p]
    L.fame_index_build.argtypes = [C.c_uint32, C.c_uint32, _P, _P, _P, C.c_int, C.c_int, _P]
    L.fame_index_build_gpu.argtypes = [C.c_uint32, C.c_uint32, _P, _P, _P, C.c_int, C.c_int, _P]
    L.fame_index_view_of.argtypes = [_P, _P]
    L.fame_index_free.argtypes = [_P]
    L.fame_index_free.restype = None
    L.fame_index_cpg_start.argtypes = [_P, _P, C.c_uint64]
    L.fame_index_cpg_start.restype = C.c_uint64
    L.fame_index_filtered_order.argtypes = [_P, _P, C.c_uint64]
    L.fame_index_filtered_order.restype = C.c_uint64
    L.fame_gpu_open.argtypes = [_P, C.c_int, _P]
    L.fame_gpu_open_layout.argtypes = [_P, C.c_int, C.c_int, _P]
    L.fame_gpu_rec_layout.argtypes = [_P, _P, _P]
    L.fame_gpu_close.argtypes = [_P]
    L.fame_gpu_last_error.argtypes = [_P]
    L.fame_gpu_last_error.restype = C.c_char_p
    L.fame_gpu_match_reads.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]
    L.fame_gpu_match_reads_dev.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P, _P]
    L.fame_gpu_tallies.argtypes = [_P, _P, C.c_int]
    L.fame_gpu_alloc.argtypes = [_P, C.c_size_t, _P]
    L.fame_gpu_free.argtypes = [_P, _P]
    L.fame_gpu_memcpy.argtypes = [_P, _P, _P, C.c_size_t, C.c_int]
    L.fame_gpu_host_alloc.argtypes = [_P, C.c_size_t, _P]
    L.fame_gpu_host_free.argtypes = [_P, _P]
    L.fame_gpu_stream.argtypes = [_P, _P]
    L.fame_gpu_set_timing.argtypes = [_P, C.c_int]
    L.fame_gpu_stage_times.argtypes = [_P, _P, C.c_int]
    L.fame_gpu_last_launches.argtypes = [_P]
    L.fame_gpu_set_seed_tier.argtypes = [_P, C.c_int]
    L.fame_gpu_autotune.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_char_p]
    L.fame_gpu_load_tuning.argtypes = [_P, C.c_char_p]
    L.fame_gpu_seed_tier_counts.argtypes = [_P, _P]
    L.fame_gpu_pair_stage_times.argtypes = [_P, _P, C.c_int]
    L.fame_gpu_map_order_probe.argtypes = [_P, _P, C.c_uint32, C.c_uint32, _P, _P]
    L.fame_gpu_index_bytes.argtypes = [_P]
    L.fame_gpu_index_bytes.restype = C.c_uint64
    L.fame_gpu_match_pairs.argtypes = [_P, _P, _P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P, _P, _P, _P]
    L.fame_gpu_match_pairs_dev.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, _P, _P, _P]
    L.fame_queue_open.argtypes = [_P, C.c_uint32, C.c_uint32, C.c_uint64, _P]
    L.fame_queue_submit.argtypes = [_P, _P, _P, C.c_uint32, C.c_uint32, _P, _P]
    L.fame_queue_ready.argtypes = [_P, C.c_int]
    L.fame_queue_wait.argtypes = [_P, C.c_int, C.c_uint32]
    L.fame_queue_collect.argtypes = [_P, C.c_int, _P, _P, _P]
    L.fame_queue_launches.argtypes = [_P]
    L.fame_queue_launches.restype = C.c_uint64
    L.fame_queue_close.argtypes = [_P]
    L.fame_gpu_tally_alloc.argtypes = [_P, _P]
    L.fame_gpu_tally_read.argtypes = [_P, _P, _P, C.c_int]
    L.fame_gpu_tally_free.argtypes = [_P, _P]
    L.fame_gpu_mem_info.argtypes = [_P, _P, _P]
    L.fame_report_cpg.argtypes = [_P, _P, C.c_char_p, C.c_int]
    L.fame_report_sc_header.argtypes = [_P, C.c_char_p]
    L.fame_report_sc_rows.argtypes = [_P, C.c_char_p, _P, C.c_char_p, C.c_int]
    L.fame_fastq_open.argtypes = [C.c_char_p, C.c_int, C.c_int, _P]
    L.fame_host_page_node.argtypes = [_P]
    L.fame_gpu_host_node.argtypes = [_P]
    L.fame_fastq_open_dev.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, _P]
    L.fame_fastq_gpu_inflate.argtypes = [_P]
    L.fame_fastq_read.argtypes = [_P, C.c_uint32, _P, C.c_uint64, _P, _P]
    L.fame_fastq_close.argtypes = [_P]
    L.fame_queue_stage.argtypes = [_P, _P, _P, _P, _P, _P]
    L.fame_queue_submit_staged.argtypes = [_P, C.c_int, C.c_uint32, C.c_uint32, _P]
    L.fame_match_fastq.argtypes = [_P, C.c_char_p, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, _P, _P, _P]
    L.fame_match_fastq_paired.argtypes = [_P, C.c_char_p, C.c_char_p, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32,
                                          C.c_int, _P, _P]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _check(rc, handle=None):
    if rc != 0:
        msg = lib().fame_gpu_last_error(handle).decode() if handle else ""
        raise FameError(rc, msg)


class HostIndex:
    """A loaded (or built) FAME index in host memory, owned by the library."""

    def __init__(self, handle):
        self.h = _P(handle) if not isinstance(handle, _P) else handle
        self.view = IndexView()
        _check(lib().fame_index_view_of(self.h, C.byref(self.view)))

    @classmethod
    def read(cls, path: str) -> "HostIndex":
        """The --load_index format (RefGenome::save / load)."""
        h = _P()
        _check(lib().fame_index_read(path.encode(), C.byref(h)))
        return cls(h)

    def write(self, path: str):
        """The --load_index format (RefGenome::save): <path> and <path>_strands."""
        _check(lib().fame_index_write(self.h, path.encode()))

    @classmethod
    def build(cls, chrom_seqs, readlen: int = 100, names=None, noloss: bool = False, threads: int = 0) -> "HostIndex":
        """Index build from chromosome sequences (uint8 arrays or bytes) on the host cores."""
        return cls._build(lib().fame_index_build, chrom_seqs, readlen, names, noloss, threads)

    @classmethod
    def build_gpu(cls, chrom_seqs, readlen: int = 100, names=None, noloss: bool = False, device: int = 0) -> "HostIndex":
        """The same index built on a GPU (identical tables)."""
        return cls._build(lib().fame_index_build_gpu, chrom_seqs, readlen, names, noloss, device)

    @classmethod
    def _build(cls, fn, chrom_seqs, readlen, names, noloss, last):
        arrs = [np.ascontiguousarray(np.frombuffer(s, np.uint8) if isinstance(s, (bytes, bytearray)) else s,
                                     dtype=np.uint8) for s in chrom_seqs]
        ptrs = (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
        lens = np.array([len(a) for a in arrs], dtype=np.uint64)
        nm = None
        if names is not None:
            enc = [n.encode() for n in names]
            nm = (C.c_char_p * len(enc))(*enc)
        h = _P()
        _check(fn(readlen, len(arrs), C.cast(ptrs, _P), _ptr(lens), C.cast(nm, _P) if nm is not None else None,
                  int(noloss), last, C.byref(h)))
        return cls(h)

    def close(self):
        if self.h:
            lib().fame_index_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- numpy views of the tables (borrowed) ----
    def _arr(self, addr, count, dtype):
        if count == 0 or not addr:
            return np.zeros(0, dtype=dtype)
        buf = (C.c_char * (int(count) * np.dtype(dtype).itemsize)).from_address(addr)
        return np.frombuffer(buf, dtype=dtype)

    @property
    def readlen(self) -> int:
        return int(self.view.readlen)

    @property
    def n_cpg(self) -> int:
        return int(self.view.n_cpg)

    def filtered_order(self):
        """filteredKmers in the order the reference's set received them."""
        n = lib().fame_index_filtered_order(self.h, None, 0)
        out = np.zeros(int(n), np.uint64)
        lib().fame_index_filtered_order(self.h, _ptr(out), n)
        return out

    def chrom_names(self):
        v = self.view
        p = C.cast(v.chrom_name, C.POINTER(C.c_char_p))
        return [p[i].decode() for i in range(v.n_chrom)]

    def chrom_seqs(self):
        v = self.view
        sp = C.cast(v.chrom_seq, C.POINTER(C.c_void_p))
        lens = self._arr(v.chrom_len, v.n_chrom, np.uint64)
        return [self._arr(sp[i], int(lens[i]), np.uint8) for i in range(v.n_chrom)]

    def tables(self, sparse: bool = True) -> dict:
        """Index tables; with sparse=True the hash-table offsets are given as the
        non-empty buckets (key, start, len), the layout of the oracle and the
        golden files, otherwise omitted (see tab_index64)."""
        v = self.view
        cpg = self._arr(v.cpg, v.n_cpg, CPG_DT)
        km = self._arr(v.kmer, v.n_kmer, KMER_DT)
        win = self._arr(v.win, v.n_win, WIN_DT)
        if sparse:
            if v.tab_index32:
                tab = self._arr(v.tab_index32, HTABSIZE + 1, np.uint32).astype(np.uint64)
            else:
                tab = self._arr(v.tab_index, HTABSIZE + 1, np.uint64)
            ln = np.diff(tab)
            keys = np.nonzero(ln)[0]
        else:
            tab = ln = keys = np.zeros(0, np.uint64)
        sbits = self._arr(v.strand_bits, (v.n_kmer + 7) // 8, np.uint8)
        strand = np.unpackbits(sbits, bitorder="little")[: v.n_kmer].astype(np.uint8)
        ncs = lib().fame_index_cpg_start(self.h, None, 0)
        cs = np.zeros(int(ncs), dtype=CPG_DT)
        lib().fame_index_cpg_start(self.h, _ptr(cs), ncs)
        return dict(cpg_chrom=np.ascontiguousarray(cpg["chrom"]), cpg_pos=np.ascontiguousarray(cpg["pos"]),
                    cpgs_chrom=np.ascontiguousarray(cs["chrom"]), cpgs_pos=np.ascontiguousarray(cs["pos"]),
                    bucket_key=keys.astype(np.uint32), bucket_start=tab[keys].astype(np.uint64),
                    bucket_len=ln[keys].astype(np.uint32), kmer_meta=np.ascontiguousarray(km["meta"]),
                    kmer_tmask=np.ascontiguousarray(km["tmask"]), strand=strand,
                    win_start=np.ascontiguousarray(win["start_pos"]), win_chrom=np.ascontiguousarray(win["chrom"]),
                    win_sind=np.ascontiguousarray(win["start_ind"]), win_eind=np.ascontiguousarray(win["end_ind"]),
                    filtered=self._arr(v.filtered, v.n_filtered, np.uint64).copy())

    def tab_index64(self):
        v = self.view
        if v.tab_index32:
            return self._arr(v.tab_index32, HTABSIZE + 1, np.uint32).astype(np.uint64)
        return self._arr(v.tab_index, HTABSIZE + 1, np.uint64)


class GpuMatcher:
    """The device context: index resident in HBM, chunk matching, tallies."""

    REC_AUTO, REC_DENSE, REC_HASHED = 0, 1, 2

    def __init__(self, index: HostIndex, device: int = 0, rec_layout: int = 0):
        """rec_layout: REC_AUTO (hashed bucket records when at most a quarter
        of the buckets are non-empty), REC_DENSE or REC_HASHED."""
        self.index = index
        self.h = _P()
        _check(lib().fame_gpu_open_layout(C.byref(index.view), device, rec_layout, C.byref(self.h)))
        self.n_cpg = index.n_cpg

    def rec_layout(self):
        """(layout, record slots, non-empty buckets) of the device index."""
        slots, nonempty = C.c_uint64(), C.c_uint64()
        layout = lib().fame_gpu_rec_layout(self.h, C.byref(slots), C.byref(nonempty))
        return layout, slots.value, nonempty.value

    def close(self):
        if self.h:
            lib().fame_gpu_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def match_reads(self, seq_bytes, offs, flags: int, mats=None, invalid=None):
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        n = len(offs) - 1
        buf = np.frombuffer(seq_bytes, dtype=np.uint8) if isinstance(seq_bytes, (bytes, bytearray)) else seq_bytes
        mats = np.zeros(n, np.uint64) if mats is None else mats
        invalid = np.zeros(n, np.uint8) if invalid is None else invalid
        cnt = Counters()
        _check(lib().fame_gpu_match_reads(self.h, _ptr(buf), _ptr(offs), n, flags, _ptr(mats), _ptr(invalid),
                                          C.byref(cnt)), self.h)
        return mats, invalid, cnt

    def match_pairs(self, seq1, offs1, seq2, offs2, flags: int, maxpdist: int):
        """One chunk of read pairs (fame_gpu_match_pairs); returns
        (mats1, mats2, invalid1, invalid2, PairCounters)."""
        offs1 = np.ascontiguousarray(offs1, dtype=np.uint64)
        offs2 = np.ascontiguousarray(offs2, dtype=np.uint64)
        n = len(offs1) - 1
        if len(offs2) != n + 1:
            raise ValueError("mate offset arrays differ in length")
        b1 = np.frombuffer(seq1, dtype=np.uint8) if isinstance(seq1, (bytes, bytearray)) else seq1
        b2 = np.frombuffer(seq2, dtype=np.uint8) if isinstance(seq2, (bytes, bytearray)) else seq2
        m1, m2 = np.zeros(n, np.uint64), np.zeros(n, np.uint64)
        i1, i2 = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
        cnt = PairCounters()
        _check(lib().fame_gpu_match_pairs(self.h, _ptr(b1), _ptr(offs1), _ptr(b2), _ptr(offs2), n, flags, maxpdist,
                                          _ptr(m1), _ptr(m2), _ptr(i1), _ptr(i2), C.byref(cnt)), self.h)
        return m1, m2, i1, i2, cnt

    def match_pairs_dev(self, seqs_dev, offs_dev, n: int, flags: int, maxpdist: int, mats_dev, invalid_dev):
        cnt = PairCounters()
        _check(lib().fame_gpu_match_pairs_dev(self.h, seqs_dev, offs_dev, n, flags, maxpdist, mats_dev, invalid_dev,
                                              C.byref(cnt)), self.h)
        return cnt

    def match_reads_dev(self, seqs_dev, offs_dev, n: int, flags: int, mats_dev, invalid_dev):
        cnt = Counters()
        _check(lib().fame_gpu_match_reads_dev(self.h, seqs_dev, offs_dev, n, flags, mats_dev, invalid_dev,
                                              C.byref(cnt)), self.h)
        return cnt

    def match_fastq(self, path: str, is_gz: bool, flags: int, chunk: int = 0, slots: int = 3, threads: int = 0,
                    meth_dev=None):
        """A whole single-end FASTQ file (fame_match_fastq): parse and match
        overlapped, strand vote on the first chunk unless FAME_BOTH_STRANDS;
        tallies accumulate in the context (or meth_dev).  Returns
        (Counters, reads)."""
        cnt = Counters()
        n = C.c_uint64(0)
        _check(lib().fame_match_fastq(self.h, path.encode(), int(is_gz), flags, chunk, slots, threads, meth_dev,
                                      C.byref(cnt), C.byref(n)), self.h)
        return cnt, int(n.value)

    def match_fastq_paired(self, path1: str, path2: str, is_gz: bool, flags: int, maxpdist: int, chunk: int = 0,
                           threads: int = 0):
        """Two mate FASTQ files (fame_match_fastq_paired): parse of the next
        chunk overlapped with the matching, strand vote on the first chunk
        unless FAME_BOTH_STRANDS; tallies accumulate in the context.  Returns
        (PairCounters, pairs)."""
        cnt = PairCounters()
        n = C.c_uint64(0)
        _check(lib().fame_match_fastq_paired(self.h, path1.encode(), path2.encode(), int(is_gz), flags, maxpdist,
                                             chunk, threads, C.byref(cnt), C.byref(n)), self.h)
        return cnt, int(n.value)

    def tallies(self, reset: bool = False) -> np.ndarray:
        out = np.empty(4 * self.n_cpg, np.uint16)
        _check(lib().fame_gpu_tallies(self.h, _ptr(out), int(reset)), self.h)
        return out.reshape(-1, 4)

    def set_timing(self, on: bool):
        _check(lib().fame_gpu_set_timing(self.h, int(on)), self.h)

    STAGES = ("read_prep", "seed", "shift_and", "select", "banded_dp", "seed_tiers", "seed_mid_small",
              "seed_mid_large", "seed_global")

    def stage_times(self):
        """fame_gpu_stage_times: per-stage milliseconds of the last single-end chunk (STAGES)."""
        ms = np.zeros(len(self.STAGES), np.float32)
        lib().fame_gpu_stage_times(self.h, _ptr(ms), len(ms))
        return ms

    def map_order_probe(self, keys, bucket_count: int):
        """fame_gpu_map_order_probe: the device replay's iteration order of distinct keys, and its final
        bucket count."""
        keys = np.ascontiguousarray(keys, dtype=np.uint32)
        order = np.zeros(max(1, len(keys)), np.uint32)
        fb = np.zeros(1, np.uint64)
        k = lib().fame_gpu_map_order_probe(self.h, _ptr(keys), len(keys), int(bucket_count), _ptr(order), _ptr(fb))
        _check(min(k, 0), self.h)
        return order[:k].copy(), int(fb[0])

    PAIR_STAGES = ("mate_checks", "seed", "seed_mid", "scans_first", "walks_first", "scans_second",
                   "walks_second_choice", "per_pair_and_dp")

    def pair_stage_times(self):
        """fame_gpu_pair_stage_times: per-stage milliseconds of the last paired chunk (PAIR_STAGES)."""
        ms = np.zeros(len(self.PAIR_STAGES), np.float32)
        lib().fame_gpu_pair_stage_times(self.h, _ptr(ms), len(ms))
        return ms

    def seed_tier_counts(self):
        """fame_gpu_seed_tier_counts: tasks entering each seeding tier after the light one, last chunk."""
        out = np.zeros(5, np.uint64)
        _check(lib().fame_gpu_seed_tier_counts(self.h, _ptr(out)), self.h)
        return out

    def last_launches(self) -> int:
        return int(lib().fame_gpu_last_launches(self.h))

    def seed_tier(self, mode: int = -1) -> int:
        """Set (0 to 3) or read (-1) the seeding mode: fame_gpu_set_seed_tier."""
        rc = lib().fame_gpu_set_seed_tier(self.h, int(mode))
        if mode >= 0:
            _check(rc, self.h)
        return rc if mode < 0 else mode

    def autotune(self, seqs_dev, offs_dev, n: int, flags: int, json_path: str) -> dict:
        """fame_gpu_autotune on a chunk in device memory; returns the JSON it wrote."""
        import json
        _check(lib().fame_gpu_autotune(self.h, seqs_dev, offs_dev, n, flags, json_path.encode()), self.h)
        with open(json_path) as f:
            return json.load(f)

    def load_tuning(self, json_path: str):
        """fame_gpu_load_tuning: apply the shapes of an autotuner file."""
        _check(lib().fame_gpu_load_tuning(self.h, json_path.encode()), self.h)

    def index_bytes(self) -> int:
        """Device bytes of the resident index tables."""
        return int(lib().fame_gpu_index_bytes(self.h))

    # device / pinned memory helpers
    def alloc(self, nbytes: int) -> int:
        p = _P()
        _check(lib().fame_gpu_alloc(self.h, nbytes, C.byref(p)), self.h)
        return p.value

    def free(self, p):
        _check(lib().fame_gpu_free(self.h, p), self.h)

    def memcpy(self, dst, src, nbytes: int, kind: int):
        _check(lib().fame_gpu_memcpy(self.h, dst, src, nbytes, kind), self.h)

    def host_alloc(self, nbytes: int) -> np.ndarray:
        p = _P()
        _check(lib().fame_gpu_host_alloc(self.h, nbytes, C.byref(p)), self.h)
        buf = (C.c_char * nbytes).from_address(p.value)
        arr = np.frombuffer(buf, dtype=np.uint8)
        return arr

    def host_free(self, arr: np.ndarray):
        _check(lib().fame_gpu_host_free(self.h, arr.ctypes.data), self.h)

    def host_node(self) -> int:
        """Host NUMA node nearest the device (-1 when unknown)."""
        return int(lib().fame_gpu_host_node(self.h))

    @staticmethod
    def page_nodes(arr: np.ndarray, samples: int = 3):
        """NUMA nodes of a few pages of a host buffer (first, middle, last)."""
        if arr.nbytes == 0:
            return []
        at = [0, arr.nbytes // 2, arr.nbytes - 1][:samples]
        return [int(lib().fame_host_page_node(C.c_void_p(arr.ctypes.data + a))) for a in at]

    # separate tally arrays (one per job of a serving loop)
    def tally_alloc(self) -> int:
        p = _P()
        _check(lib().fame_gpu_tally_alloc(self.h, C.byref(p)), self.h)
        return p.value

    def tally_read(self, meth_dev: int, reset: bool = False) -> np.ndarray:
        out = np.empty(4 * self.n_cpg, np.uint16)
        _check(lib().fame_gpu_tally_read(self.h, meth_dev, _ptr(out), int(reset)), self.h)
        return out.reshape(-1, 4)

    def tally_free(self, meth_dev: int):
        _check(lib().fame_gpu_tally_free(self.h, meth_dev), self.h)

    def mem_info(self):
        f, t = C.c_uint64(), C.c_uint64()
        _check(lib().fame_gpu_mem_info(self.h, C.byref(f), C.byref(t)), self.h)
        return f.value, t.value


class FastqReader:
    """Native FASTQ chunk reader (fame_fastq_*): parseChunk's records, the
    sequences packed with offsets, into page-locked buffers when given."""

    def __init__(self, path: str, is_gz: bool = False, n_threads: int = 0, max_reads: int = 300000,
                 max_len: int = 256, seqs: np.ndarray = None, offs: np.ndarray = None, device: int = -1):
        """device >= 0: BGZF input is inflated on that GPU (fame_fastq_open_dev)."""
        self.h = _P()
        _check(lib().fame_fastq_open_dev(path.encode(), int(is_gz), n_threads, device, C.byref(self.h)))
        self.max_reads = max_reads
        self.seqs = np.zeros(max_reads * max_len, np.uint8) if seqs is None else seqs
        self.offs = np.zeros(max_reads + 1, np.uint64) if offs is None else offs

    def read(self):
        """Next chunk: (sequence bytes view, offsets view) of n records (n == 0 at the end)."""
        n = C.c_uint32()
        _check(lib().fame_fastq_read(self.h, self.max_reads, _ptr(self.seqs), self.seqs.nbytes, _ptr(self.offs),
                                     C.byref(n)))
        k = n.value
        return self.seqs[: int(self.offs[k])], self.offs[: k + 1]

    @property
    def gpu_inflate(self) -> bool:
        """True when the input is inflated on a GPU (BGZF)."""
        return bool(lib().fame_fastq_gpu_inflate(self.h))

    def close(self):
        if self.h:
            lib().fame_fastq_close(self.h)
            self.h = None


class GpuQueue:
    """The batched form (fame_queue_*): chunk slots on a GpuMatcher's context,
    each running the chunk pipeline as a CUDA graph on its own stream."""

    def __init__(self, gpu: GpuMatcher, slots: int, max_reads: int, max_bytes: int):
        self.gpu = gpu
        self.nslots = slots
        self.h = _P()
        _check(lib().fame_queue_open(gpu.h, slots, max_reads, max_bytes, C.byref(self.h)), gpu.h)
        self.pending = {}

    def submit(self, seq_bytes, offs, flags: int, meth_dev=None) -> int:
        offs = np.ascontiguousarray(offs, dtype=np.uint64)
        n = len(offs) - 1
        buf = np.frombuffer(seq_bytes, dtype=np.uint8) if isinstance(seq_bytes, (bytes, bytearray)) else seq_bytes
        slot = C.c_int()
        _check(lib().fame_queue_submit(self.h, _ptr(buf), _ptr(offs), n, flags, meth_dev, C.byref(slot)), self.gpu.h)
        self.pending[slot.value] = n
        return slot.value

    def ready(self, slot: int) -> bool:
        return lib().fame_queue_ready(self.h, slot) == 1

    def wait(self, slot: int, timeout_ms: int) -> bool:
        """True when the slot's chunk finished within timeout_ms, False when the
        wait timed out (FAME_ERR_TIMEOUT); other errors raise."""
        rc = lib().fame_queue_wait(self.h, slot, int(timeout_ms))
        if rc == -7:
            return False
        _check(rc, self.gpu.h)
        return True

    def collect(self, slot: int, mats=None, invalid=None):
        n = self.pending.pop(slot)
        mats = np.zeros(n, np.uint64) if mats is None else mats
        invalid = np.zeros(n, np.uint8) if invalid is None else invalid
        cnt = Counters()
        _check(lib().fame_queue_collect(self.h, slot, _ptr(mats), _ptr(invalid), C.byref(cnt)), self.gpu.h)
        return mats, invalid, cnt

    def launches(self) -> int:
        return int(lib().fame_queue_launches(self.h))

    def close(self):
        if self.h and self.gpu.h:          # closing the context closes its queue
            lib().fame_queue_close(self.h)
        self.h = None
