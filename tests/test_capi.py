"""The C ABI library: it builds, loads, exports every declared entry point and
reports argument and I/O errors (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

from fame_gb300 import _lib
from fame_gb300 import build as fbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fame_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|uint64_t)\s+(fame_\w+)\s*\(", src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert os.path.exists(fbuild.LIB)


def test_argument_errors_without_gpu():
    L = _lib.lib()
    assert L.fame_gpu_open(None, 0, None) == -1
    assert L.fame_gpu_close(None) == -1
    assert L.fame_gpu_match_reads(None, None, None, 0, 0, None, None, None) == -1
    assert L.fame_gpu_tallies(None, None, 0) == -1
    assert L.fame_index_read(None, None) == -1
    assert L.fame_gpu_match_pairs(None, None, None, None, None, 0, 0, 550, None, None, None, None, None) == -1
    assert L.fame_gpu_match_pairs_dev(None, None, None, 0, 0, 550, None, None, None) == -1
    assert L.fame_queue_open(None, 2, 10, 1000, None) == -1
    assert L.fame_queue_submit(None, None, None, 0, 0, None, None) == -1
    assert L.fame_queue_collect(None, 0, None, None, None) == -1
    assert L.fame_queue_ready(None, 0) == -1
    assert L.fame_queue_close(None) == -1
    assert L.fame_gpu_tally_alloc(None, None) == -1
    assert L.fame_gpu_tally_read(None, None, None, 0) == -1
    assert L.fame_gpu_mem_info(None, None, None) == -1
    assert L.fame_queue_stage(None, None, None, None, None, None) == -1
    assert L.fame_queue_submit_staged(None, 0, 0, 0, None) == -1
    assert L.fame_match_fastq(None, b"x.fq", 0, 0, 0, 2, 0, None, None, None) == -1
    assert L.fame_match_fastq_paired(None, b"1.fq", b"2.fq", 0, 0, 550, 0, 0, None, None) == -1
    assert L.fame_index_write(None, b"x.idx") == -1
    # entry points of the device layouts, the device index build and reader, the diagnostics
    assert L.fame_gpu_open_layout(None, 0, 0, None) == -1
    assert L.fame_gpu_rec_layout(None, None, None) == -1
    assert L.fame_index_build_gpu(100, 0, None, None, None, 0, 0, None) == -1
    assert L.fame_fastq_open_dev(None, 1, 0, 0, None) == -1
    assert L.fame_fastq_gpu_inflate(None) == 0
    assert L.fame_index_filtered_order(None, None, 0) == 0
    assert L.fame_host_page_node(None) == -1
    assert L.fame_gpu_host_node(None) == -1


def test_open_layout_rejects_unknown_layouts(product_index):
    """An unknown record layout is an argument error, before any device call."""
    import ctypes
    L = _lib.lib()
    h = ctypes.c_void_p()
    for layout in (-1, 3, 99):
        assert L.fame_gpu_open_layout(ctypes.byref(product_index.view), 0, layout, ctypes.byref(h)) == -1


def test_index_read_errors(tmp_path):
    L = _lib.lib()
    h = C.c_void_p()
    assert L.fame_index_read(str(tmp_path / "missing.idx").encode(), C.byref(h)) == -6
    bad = tmp_path / "bad.idx"
    bad.write_bytes(b"\x00" * 64)   # wrong HTABSIZE in the header
    assert L.fame_index_read(str(bad).encode(), C.byref(h)) == -6
    import struct
    hdr = struct.pack("<QIIIQI", 1 << 30, 100, 2048, 32, 1500, 0xDEFDFFFD)
    trunc = tmp_path / "trunc.idx"
    trunc.write_bytes(hdr + struct.pack("<Q", 5))   # announces 5 CpGs, ends there
    assert L.fame_index_read(str(trunc).encode(), C.byref(h)) == -6
    huge = tmp_path / "huge.idx"
    huge.write_bytes(hdr + struct.pack("<Q", 1 << 62))   # a CpG count no file can hold
    assert L.fame_index_read(str(huge).encode(), C.byref(h)) in (-3, -6)
    wrongseed = tmp_path / "seed.idx"
    wrongseed.write_bytes(struct.pack("<QIIIQI", 1 << 30, 100, 2048, 32, 1500, 0x12345678))
    assert L.fame_index_read(str(wrongseed).encode(), C.byref(h)) == -6


def test_lib_rebuild_is_noop_when_fresh():
    fbuild.build()
    assert fbuild.up_to_date()
