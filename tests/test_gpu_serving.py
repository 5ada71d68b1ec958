"""The serving loop (fame_gb300/serving.py) over the batched queue: jobs of
very different sizes admitted while others run, their chunks interleaved in
the queue's slots; every job's matches, counters and CpG tallies equal the
job run alone through the plain chunk calls (single-cell semantics: its own
strand vote and tallies)."""
import numpy as np
import pytest

from fame_gb300 import GpuMatcher
from fame_gb300.serving import Job, ServingLoop, latency_summary, plain_per_job

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(product_index):
    g = GpuMatcher(product_index, 0)
    yield g
    g.close()


def golden_jobs(golden, sizes):
    seq = golden["read_seq"].tobytes()
    offs = golden["read_offs"]
    jobs, a = [], 0
    for i, n in enumerate(sizes):
        o = offs[a:a + n + 1].astype(np.uint64)
        jobs.append(Job("cell%d" % i, seq[int(o[0]):int(o[-1])], o - o[0], arrival=0.001 * i))
        a += n
    return jobs


def same(a, b):
    assert a.job_id == b.job_id
    assert np.array_equal(a.mats, b.mats) and np.array_equal(a.invalid, b.invalid), a.job_id
    assert a.counters == b.counters, (a.job_id, a.counters, b.counters)
    assert np.array_equal(a.meth, b.meth), a.job_id


@pytest.mark.parametrize("realtime", [False, True], ids=["burst", "arrivals"])
def test_jobs_same_alone_and_mixed(gpu, golden, realtime):
    sizes = [1700, 40, 900, 2200, 300, 866]           # 6,006 reads, chunks of 500
    jobs = golden_jobs(golden, sizes)
    ref = {r.job_id: r for r in plain_per_job(gpu, jobs, chunk=500, realtime=False)}
    loop = ServingLoop(gpu, slots=3, chunk=500, max_active=4)
    try:
        mixed = loop.run(jobs, realtime=realtime)
        alone = [loop.run([j], realtime=False)[0] for j in jobs[:2]]
    finally:
        loop.close()
    assert sorted(r.job_id for r in mixed) == sorted(ref)
    for r in mixed + alone:
        same(r, ref[r.job_id])
    s = latency_summary(mixed)
    assert s["jobs"] == len(jobs) and s["p99_ms"] >= s["p50_ms"] > 0
