"""GB300-native read matching for the FAME bisulfite aligner.

The product is the native library ``libfame_gpu.so`` (CUDA kernels for
sm_103a and host C++ behind the C ABI in ``include/fame_gpu.h``); this
package holds its sources (``csrc/``), the in-tree build, a ctypes binding
and a host-side mirror of FAME's ReadQueue interface.
"""
from ._lib import (CHUNKSIZE, FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, FAME_MAX_READ_LEN,
                   Counters, FameError, GpuMatcher, GpuQueue, HostIndex, PairCounters, lib)
from .readqueue import PairedReadQueue, ReadQueue, SingleCellQueue, read_sc_meta, write_cpg_report
from . import synth

__all__ = ["CHUNKSIZE", "FAME_BOTH_STRANDS", "FAME_GET_STRANDED", "FAME_MATCH_R1_FWD", "FAME_MAX_READ_LEN",
           "Counters", "FameError", "GpuMatcher", "GpuQueue", "HostIndex", "PairCounters", "lib", "PairedReadQueue", "ReadQueue", "SingleCellQueue", "read_sc_meta", "write_cpg_report"]
