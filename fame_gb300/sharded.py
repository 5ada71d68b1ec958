"""Read-sharded matching over several processes (one GPU each).

Reads are independent in FAME's matching stage, so chunks shard across ranks
with no data-path collective.  Two pieces of state are global in the
reference and are exchanged here (torch.distributed, any backend):

* the strand vote of the first chunk (r1FwdMatches / r1RevMatches,
  ReadQueue.cpp:376-400): every rank matches its slice of chunk 0 with
  getStranded, the votes are summed, and all ranks take the same decision;
* the CpG tallies (methLevels, ReadQueue.h:354-367): summed element-wise at
  the end; uint16 wrap-around commutes with the sum, so the result equals a
  single process's tallies.

Chunk c >= 1 goes to rank c % world.  `matcher` is any object with
match(seq_bytes, offs, flags) -> (mats, invalid, counters) and
tallies(reset) -> uint16 array (GpuMatcher on a GPU).
"""
from __future__ import annotations

import numpy as np

from ._lib import CHUNKSIZE, FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD


def _allreduce_sum(arr: np.ndarray, dist) -> np.ndarray:
    import torch
    t = torch.from_numpy(np.ascontiguousarray(arr.astype(np.int64)))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.numpy()


def sharded_query(seq: bytes, offs: np.ndarray, matcher, rank: int, world: int, dist=None,
                  chunk: int = CHUNKSIZE, both_strands: bool = False):
    """queryRoutine (main.cpp:363-399) over `world` ranks.

    Returns (read_ids, mats, invalid) for the reads this rank matched, and the
    reduced (uint16 tallies, counters [succ, nonunique, unsucc, r1Fwd, r1Rev,
    matchR1Fwd]) that are identical on every rank."""
    n = len(offs) - 1
    chunks = [(c0, min(n, c0 + chunk)) for c0 in range(0, n, chunk)] or [(0, 0)]
    ids, mats_all, inv_all = [], [], []
    cnt = np.zeros(5, np.int64)
    match_r1_fwd = True

    def run(a, b, flags):
        o = offs[a:b + 1].astype(np.uint64)
        m, iv, c = matcher.match(seq[int(o[0]):int(o[-1])], o - o[0], flags)
        ids.append(np.arange(a, b, dtype=np.int64))
        mats_all.append(m)
        inv_all.append(iv)
        cnt[:] += np.array([c[0], c[1], c[2], c[3], c[4]], dtype=np.int64)

    first = 0
    if not both_strands:
        a, b = chunks[0]
        per = (b - a + world - 1) // world
        sa, sb = min(b, a + rank * per), min(b, a + (rank + 1) * per)
        if sb > sa:
            run(sa, sb, FAME_GET_STRANDED)
        votes = cnt[3:5].copy()
        if dist is not None and world > 1:
            votes = _allreduce_sum(votes, dist)
        match_r1_fwd = bool(votes[0] > votes[1])
        cnt[3:5] = 0
        first = 1
        tot_votes = votes
    else:
        tot_votes = np.zeros(2, np.int64)
    for ci in range(first, len(chunks)):
        if ci % world != rank:
            continue
        a, b = chunks[ci]
        if b > a:
            flags = (FAME_BOTH_STRANDS if both_strands else 0) | (FAME_MATCH_R1_FWD if match_r1_fwd else 0)
            run(a, b, flags)
    meth = matcher.tallies(reset=True).astype(np.int64)
    if dist is not None and world > 1:
        meth = _allreduce_sum(meth, dist)
        cnt = _allreduce_sum(cnt, dist)
    meth = (meth & 0xFFFF).astype(np.uint16)
    counters = np.array([cnt[0], cnt[1], cnt[2], tot_votes[0], tot_votes[1], int(match_r1_fwd)], dtype=np.uint64)
    cat = (lambda xs, dt: np.concatenate(xs) if xs else np.zeros(0, dt))
    return (cat(ids, np.int64), cat(mats_all, np.uint64), cat(inv_all, np.uint8)), meth, counters


class GpuShardMatcher:
    """Adapter of GpuMatcher to the matcher interface of sharded_query."""

    def __init__(self, gpu):
        self.gpu = gpu

    def match(self, seq_bytes, offs, flags):
        m, iv, c = self.gpu.match_reads(seq_bytes, offs, flags)
        return m, iv, (c.succ, c.nonunique, c.unsucc, c.r1_fwd, c.r1_rev)

    def tallies(self, reset=True):
        return self.gpu.tallies(reset=reset)
