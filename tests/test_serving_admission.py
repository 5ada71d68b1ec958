"""Admission control of the serving loop, on the host (no GPU): the device is a
fake whose free memory and tally allocations the test sets.

* A job whose tally array does not fit waits while other jobs run and is
  admitted when they free theirs.
* With nothing running, a job that does not fit can never be admitted: it is
  refused (its result says why) and the loop goes on with the next job.
* A tally allocation that fails with FAME_ERR_NOMEM (the host-side image of
  a failed cudaMalloc) is treated the same way.
"""
import numpy as np

from fame_gb300._lib import FameError
from fame_gb300.serving import Job, ServingLoop


class FakeCounters:
    def __init__(self, n):
        self.succ, self.nonunique, self.unsucc, self.r1_fwd, self.r1_rev = n, 0, 0, n, 0


class FakeQueue:
    """Chunks finish when collected; results: every read matched."""

    def __init__(self, nslots=2):
        self.nslots = nslots
        self.busy = {}
        self.order = []

    def submit(self, seq, offs, flags, tally):
        s = next(i for i in range(self.nslots) if i not in self.busy)
        self.busy[s] = (len(offs) - 1, tally)
        self.order.append(tally)
        return s

    def ready(self, slot):
        return True

    def collect(self, slot):
        n, _ = self.busy.pop(slot)
        return np.zeros(n, np.uint64), np.zeros(n, np.uint8), FakeCounters(n)

    def close(self):
        pass


class FakeGpu:
    """Free device memory shrinks by a tally array per admitted job; tally
    allocations fail while fail_allocs > 0."""

    n_cpg = 1000

    def __init__(self, free, fail_allocs=0):
        self.free = free
        self.fail_allocs = fail_allocs
        self.live = set()
        self.next = 1

    def mem_info(self):
        return self.free, 1 << 40

    def tally_alloc(self):
        if self.fail_allocs > 0:
            self.fail_allocs -= 1
            raise FameError(-3, "device allocation of 16000 bytes failed")
        t = self.next
        self.next += 1
        self.live.add(t)
        self.free -= 16 * self.n_cpg
        return t

    def tally_read(self, t):
        return np.zeros((self.n_cpg, 4), np.uint16)

    def tally_free(self, t):
        self.live.remove(t)
        self.free += 16 * self.n_cpg


def jobs(n, reads=10):
    out = []
    for i in range(n):
        offs = np.arange(reads + 1, dtype=np.uint64) * 100
        out.append(Job("job%d" % i, b"A" * (100 * reads), offs, arrival=0.0))
    return out


def loop(gpu, reserve, chunk=4):
    return ServingLoop(gpu, chunk=chunk, mem_reserve=reserve, queue=FakeQueue())


def test_jobs_wait_for_memory_and_are_admitted():
    # room for one tally array above the reserve at a time: jobs run one after another
    gpu = FakeGpu(free=16_000 + 1_000 + 1)
    res = loop(gpu, reserve=1_000).run(jobs(3), realtime=False)
    assert [r.status for r in res] == ["ok"] * 3
    assert sorted(r.job_id for r in res) == ["job0", "job1", "job2"]
    assert all(r.counters["succ"] == 10 for r in res)
    assert not gpu.live


def test_job_that_can_never_fit_is_refused():
    gpu = FakeGpu(free=500)
    res = loop(gpu, reserve=1_000).run(jobs(2), realtime=False)
    assert len(res) == 2
    assert all(r.status.startswith("refused: device memory") for r in res)
    assert all(r.meth is None for r in res)
    assert not gpu.live


def test_failed_tally_allocation_waits_or_refuses():
    # the first allocation fails with nothing running: that job is refused,
    # the next ones are admitted
    gpu = FakeGpu(free=1 << 30, fail_allocs=1)
    res = loop(gpu, reserve=0).run(jobs(3), realtime=False)
    st = {r.job_id: r.status for r in res}
    assert st["job0"].startswith("refused: tally allocation failed")
    assert st["job1"] == "ok" and st["job2"] == "ok"
    # with a job running, a failed allocation only makes the next job wait
    gpu = FakeGpu(free=1 << 30)
    sl = loop(gpu, reserve=0)
    orig = gpu.tally_alloc
    calls = {"n": 0}

    def flaky():
        calls["n"] += 1
        if calls["n"] == 2:
            raise FameError(-3, "device allocation failed")
        return orig()

    gpu.tally_alloc = flaky
    res = sl.run(jobs(3), realtime=False)
    assert [r.status for r in res] == ["ok"] * 3
    assert not gpu.live


def test_other_errors_propagate():
    gpu = FakeGpu(free=1 << 30)

    def broken():
        raise FameError(-2, "cuda failure")

    gpu.tally_alloc = broken
    try:
        loop(gpu, reserve=0).run(jobs(1), realtime=False)
    except FameError as e:
        assert e.code == -2
    else:
        raise AssertionError("a CUDA error must not be taken for a full device")
