"""Serving form: a request loop for single-cell-like jobs on one GPU.

Jobs (one cell's reads each, of very different sizes) arrive over time.  A
job is admitted when a tally array for it fits in free device memory (the
index stays resident) and fewer than `max_active` jobs are running; its reads
are cut into chunks that run in the batched queue's slots (fame_queue_*),
interleaved with the chunks of every other admitted job, so jobs that arrive
while others are on the GPU start at once and their work overlaps on the
device.  Per job the reference's single-cell semantics hold
(matchSCBatch, ReadQueue.cpp:1660-1748): its first chunk runs with
getStranded and its own strand vote decides the orientation of its later
chunks, and its CpG tallies are its own array.  So a job's result is the same
alone and in the mix (tests/test_gpu_serving.py).

`plain_per_job` is the comparison: each job runs by itself through the plain
chunk calls, in arrival order, as soon as the previous one is done.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import CHUNKSIZE, FAME_BOTH_STRANDS, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, FameError, GpuMatcher, GpuQueue

FAME_ERR_NOMEM = -3


@dataclass
class Job:
    job_id: str
    seq: bytes
    offs: np.ndarray          # uint64, n + 1
    arrival: float = 0.0      # seconds after the loop starts

    @property
    def n_reads(self) -> int:
        return len(self.offs) - 1


@dataclass
class JobResult:
    job_id: str
    n_reads: int
    meth: np.ndarray          # uint16 tallies, 4 per CpG
    counters: dict
    mats: np.ndarray
    invalid: np.ndarray
    arrival: float
    admitted: float
    finished: float
    status: str = "ok"        # "refused: <why>" when the job could not be admitted at all

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


@dataclass
class _Active:
    job: Job
    tally: int
    admitted: float
    chunks: list
    next_chunk: int = 0
    collected: int = 0
    flags: int = 0
    first_done: bool = False
    inflight: int = 0
    mats: np.ndarray = None
    invalid: np.ndarray = None
    counters: dict = field(default_factory=lambda: dict(succ=0, nonunique=0, unsucc=0, r1_fwd=0, r1_rev=0))


def _chunks(n, chunk):
    return [(a, min(n, a + chunk)) for a in range(0, n, chunk)] or [(0, 0)]


class ServingLoop:
    def __init__(self, gpu: GpuMatcher, slots: int = 4, chunk: int = CHUNKSIZE, max_active: int = 16,
                 both_strands: bool = False, max_bytes_per_read: int = 256, mem_reserve: int = 2 << 30,
                 queue=None):
        self.gpu = gpu
        self.chunk = chunk
        self.max_active = max_active
        self.both = both_strands
        self.mem_reserve = mem_reserve
        self.queue = queue if queue is not None else GpuQueue(gpu, slots, chunk, chunk * max_bytes_per_read)
        self.tally_bytes = 16 * max(1, gpu.n_cpg)

    def close(self):
        self.queue.close()

    def _admissible(self):
        """None when a job's tally array fits in free device memory above the
        reserve, else the reason it does not."""
        free, _ = self.gpu.mem_info()
        need = self.tally_bytes + self.mem_reserve
        return None if free > need else "device memory: %d bytes free, %d needed" % (free, need)

    def run(self, jobs, realtime: bool = True):
        """Serve `jobs` (arrival times in seconds from now when realtime, else
        all at once); returns the JobResults in completion order."""
        pending = sorted(jobs, key=lambda j: j.arrival)
        active: list[_Active] = []
        slots = {}               # slot -> (active, chunk index)
        done = []
        t0 = time.perf_counter()
        q = self.queue

        def now():
            return time.perf_counter() - t0

        while pending or active:
            t = now()
            # admission: arrived jobs, while device memory and the active limit
            # allow.  A job that does not fit waits for running jobs to free
            # their tallies; with none running it can never fit and is refused.
            while pending and (not realtime or pending[0].arrival <= t) and len(active) < self.max_active:
                why = self._admissible()
                tally = None
                if why is None:
                    try:
                        tally = self.gpu.tally_alloc()
                    except FameError as e:
                        if e.code != FAME_ERR_NOMEM:
                            raise
                        why = "tally allocation failed: %s" % e
                if tally is None:
                    if not active:
                        job = pending.pop(0)
                        n = job.n_reads
                        done.append(JobResult(job.job_id, n, None, dict(succ=0, nonunique=0, unsucc=0, r1_fwd=0,
                                                                        r1_rev=0), np.zeros(n, np.uint64),
                                              np.zeros(n, np.uint8), job.arrival, t, now(),
                                              status="refused: " + why))
                        continue
                    break
                job = pending.pop(0)
                n = job.n_reads
                active.append(_Active(job=job, tally=tally, admitted=t,
                                      chunks=_chunks(n, self.chunk), mats=np.zeros(n, np.uint64),
                                      invalid=np.zeros(n, np.uint8),
                                      flags=FAME_BOTH_STRANDS if self.both else FAME_GET_STRANDED))
            # fill free slots, oldest job first; a job's later chunks wait for its strand vote
            progressed = False
            for a in active:
                while len(slots) < q.nslots and a.next_chunk < len(a.chunks):
                    if a.next_chunk > 0 and not a.first_done and not self.both:
                        break
                    c0, c1 = a.chunks[a.next_chunk]
                    o = a.job.offs[c0:c1 + 1].astype(np.uint64)
                    s = q.submit(a.job.seq[int(o[0]):int(o[-1])], o - o[0], a.flags, a.tally)
                    slots[s] = (a, a.next_chunk)
                    a.next_chunk += 1
                    a.inflight += 1
                    progressed = True
                if len(slots) >= q.nslots:
                    break
            # collect finished chunks (the oldest submission blocks when nothing else can move)
            ready = [s for s in list(slots) if q.ready(s)]
            if not ready and slots and not progressed and (not pending or not realtime or pending[0].arrival > now()):
                ready = [next(iter(slots))]
            for s in ready:
                a, ci = slots.pop(s)
                c0, c1 = a.chunks[ci]
                m, iv, c = q.collect(s)
                a.mats[c0:c1], a.invalid[c0:c1] = m, iv
                for k in a.counters:
                    a.counters[k] += getattr(c, k)
                a.inflight -= 1
                a.collected += 1
                if ci == 0 and not self.both:
                    a.first_done = True
                    a.flags = FAME_MATCH_R1_FWD if a.counters["r1_fwd"] > a.counters["r1_rev"] else 0
            for a in [a for a in active if a.collected == len(a.chunks)]:
                meth = self.gpu.tally_read(a.tally)
                self.gpu.tally_free(a.tally)
                active.remove(a)
                done.append(JobResult(a.job.job_id, a.job.n_reads, meth, dict(a.counters), a.mats, a.invalid,
                                      a.job.arrival, a.admitted, now()))
            if not active and pending and realtime:
                wait = pending[0].arrival - now()
                if wait > 0:
                    time.sleep(min(wait, 0.002))
        return done


def plain_per_job(gpu: GpuMatcher, jobs, chunk: int = CHUNKSIZE, both_strands: bool = False, realtime: bool = True):
    """Each job alone through the plain chunk calls (fame_gpu_match_reads), in
    arrival order, with the context's tallies read and reset per job."""
    out = []
    t0 = time.perf_counter()
    for job in sorted(jobs, key=lambda j: j.arrival):
        if realtime:
            while time.perf_counter() - t0 < job.arrival:
                time.sleep(0.0005)
        start = time.perf_counter() - t0
        n = job.n_reads
        mats = np.zeros(n, np.uint64)
        inval = np.zeros(n, np.uint8)
        cnt = dict(succ=0, nonunique=0, unsucc=0, r1_fwd=0, r1_rev=0)
        flags = FAME_BOTH_STRANDS if both_strands else FAME_GET_STRANDED
        gpu.tallies(reset=True)
        for ci, (c0, c1) in enumerate(_chunks(n, chunk)):
            o = job.offs[c0:c1 + 1].astype(np.uint64)
            m, iv, c = gpu.match_reads(job.seq[int(o[0]):int(o[-1])], o - o[0], flags)
            mats[c0:c1], inval[c0:c1] = m, iv
            for k in cnt:
                cnt[k] += getattr(c, k)
            if ci == 0 and not both_strands:
                flags = FAME_MATCH_R1_FWD if cnt["r1_fwd"] > cnt["r1_rev"] else 0
        meth = gpu.tallies(reset=True)
        out.append(JobResult(job.job_id, n, meth, cnt, mats, inval, job.arrival, start, time.perf_counter() - t0))
    return out


def latency_summary(results):
    results = [r for r in results if r.status == "ok"]
    lat = np.array([r.latency for r in results]) if results else np.zeros(1)
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "jobs": len(results)}
