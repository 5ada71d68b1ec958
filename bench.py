"""Benchmark: aligned reads/s of FAME's matching stage on one GB300.

Default workload (se150_uneven_3gbp): a 24-chromosome, 3.0 Gbp synthetic
genome with 45 % interspersed repeats and 20M single-end bisulfite reads of
uneven trimmed length (60 % at 150 bp, 40 % uniform in 36-149 bp; 0.5-2 %
errors per read; 5 % of the reads drawn from repeat copies), READLEN 150,
seeded (fame_gb300/synth.py).  One step = one CHUNKSIZE (300,000 read) chunk
through ReadQueue::matchReads semantics on the GPU: seeding and index
gathers, Shift-And over every candidate window, uniqueness selection, banded
DP and CpG tallies.  The first chunk (both orientations, strand vote) runs in
the warm-up; timed steps are the following chunks in the decided
orientation, as FAME's queryRoutine runs them.

value:    reads/s of the plain form with the reads resident in HBM
          (fame_gpu_match_reads_dev), CUDA events on the library's stream.
e2e:      reads/s through fame_gpu_match_reads from page-locked host buffers,
          host-to-device copy of the chunk and device-to-host copy of the
          results inside the timed region.
batched:  the same chunks through the batched form (fame_queue_*: chunk slots
          as CUDA graphs on their own streams) from the same host buffers.
parity:   the reference's own matchReads (compiled from its sources,
          oracle/_ref) on a sample of chunk 1, compared read by read and CpG by
          CpG with the GPU's output for the same reads.
Every step gathers from a device index of tens of GB and new reads: inputs
far larger than the 129 MB L2.

--workload pe100_3gbp: paired-end (20M pairs of 2 x 100 bp, MAXPDIST 400).
--workload sc_serving: the serving form.
--impl reference: the reference's own OpenMP matchReads / matchPairedReads on
the machine's host cores, on bounded samples of the same chunks.
"""
from __future__ import annotations

import argparse
import ctypes
import gc
import hashlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "aligned reads/s (single-end matching stage, bit-exact CpG report)"
PE_METRIC = "aligned read pairs/s (paired-end matching stage, bit-exact CpG report)"
DEFAULT_WORKLOAD = "se150_uneven_3gbp"

# Sources of the kernels whose ncu figures are quoted below; a figure is
# reported only while the hash of these files equals the one it was captured with.
KERNEL_SOURCES = ("fame_gb300/csrc/seed.cuh", "fame_gb300/csrc/kernels.cuh", "fame_gb300/csrc/dev_common.cuh",
                  "fame_gb300/csrc/seedhash.h", "fame_gb300/csrc/qgram.h", "fame_gb300/csrc/editscan.h")
# ncu figures per workload: DRAM bytes (read + write) of the seeding launches
# of one steady-state chunk and the ALU-pipe utilisation of the two ALU-bound
# kernels, with the source hash and the profile that holds the capture command.
NCU_FIGURES = {
    "se150_uneven_3gbp": {"source_hash": "7a95f144a54c9c1d", "seed_traffic_per_step": 3300354048,
                          "shiftand_alu": 0.5601, "dp_alu": 0.7051,
                          "profile": "profiles/seeding_se150_uneven_3gbp.md"},
}


def kernel_source_hash() -> str:
    h = hashlib.sha256()
    for p in KERNEL_SOURCES:
        with open(os.path.join(ROOT, p), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=12)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default=DEFAULT_WORKLOAD)
    p.add_argument("--reads", type=int, default=0, help="override the workload's read (pair) count")
    p.add_argument("--cpu-sample", type=int, default=60000, help="reads (pairs) of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fastq", action="store_true", help="skip the whole-file leg")
    p.add_argument("--index-build", default="gpu", choices=["gpu", "host"],
                   help="where the GB300 arms build the index (identical tables either way)")
    p.add_argument("--index-check", action="store_true",
                   help="build the index both ways, time both and compare every table")
    return p.parse_args()


def build_index(args, seqs, readlen, device):
    """The index for a GB300 arm: fame_index_build_gpu (default) or the
    host build; with --index-check both, timed, every table compared.
    Returns (index, seconds, report)."""
    from fame_gb300 import HostIndex
    gpu_first = args.index_build == "gpu"

    def one(on_gpu):
        t0 = time.time()
        hi = (HostIndex.build_gpu(seqs, readlen=readlen, device=device) if on_gpu
              else HostIndex.build(seqs, readlen=readlen, threads=0))
        return hi, time.time() - t0

    try:
        hi, t = one(gpu_first)
        rep = {"where": args.index_build, "seconds": t}
    except Exception as e:   # setup only: the host build gives the same tables
        if not gpu_first:
            raise
        hi, t = one(False)
        rep = {"where": "host", "seconds": t, "device_build_failed": str(e)[:200]}
        gpu_first = False
    if args.index_check and "device_build_failed" not in rep:
        other, t2 = one(not gpu_first)
        rep["gpu_seconds"], rep["host_seconds"] = (t, t2) if gpu_first else (t2, t)
        rep["host_threads"] = os.cpu_count()
        rep["identical"] = same_index(hi, other)
        other.close()
    return hi, t, rep


def same_index(a, b):
    """Every table of two host indexes equal (bucket offsets, entries, T
    masks, strandTable, windows, CpGs, filtered k-mers and their order)."""
    import numpy as np
    from fame_gb300._lib import HTABSIZE
    ta, tb = a.tables(sparse=False), b.tables(sparse=False)
    if any(not np.array_equal(ta[k], tb[k]) for k in ta):
        return False
    o32 = [x._arr(x.view.tab_index32, HTABSIZE + 1, np.uint32) for x in (a, b)]
    return bool(np.array_equal(o32[0], o32[1]) and np.array_equal(a.filtered_order(), b.filtered_order()))


# ---------------------------------------------------------------------------
def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


_REAL_STDOUT = None


def stdout_to_stderr():
    """The bench's only stdout is its JSON line: everything else written to
    file descriptor 1 (the reference library's C++ output included) goes to
    stderr."""
    global _REAL_STDOUT
    sys.stdout.flush()
    _REAL_STDOUT = os.fdopen(os.dup(1), "w")
    os.dup2(2, 1)


def emit(obj):
    """Write the JSON line to the real stdout, after flushing C stdio."""
    try:
        ctypes.CDLL(None).fflush(None)
    except Exception:
        pass
    sys.stdout.flush()
    out = _REAL_STDOUT or sys.stdout
    out.write(json.dumps(obj) + "\n")
    out.flush()


def host_placement(device):
    """Host facts that bound the end-to-end copies: the GPU's nearest host NUMA
    node (sysfs, by PCI bus id) and the memory nodes / CPUs this process may use.
    Page-locked buffers go to the GPU's node when the process may use it."""
    out = {}
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(device), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=30).stdout.strip()
        dom, rest = bus.split(":", 1)
        with open("/sys/bus/pci/devices/%04x:%s/numa_node" % (int(dom, 16), rest.lower())) as f:
            out["gpu_host_numa_node"] = int(f.read().strip())
    except Exception:
        out["gpu_host_numa_node"] = None
    try:
        with open("/proc/self/status") as f:
            for line in f:
                if line.startswith("Mems_allowed_list:"):
                    out["mems_allowed"] = line.split(":", 1)[1].strip()
                if line.startswith("Cpus_allowed_list:"):
                    out["cpus_allowed"] = line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:   # free memory per host node at the time of the call
        import glob
        free = {}
        for path in sorted(glob.glob("/sys/devices/system/node/node*/meminfo")):
            with open(path) as f:
                for line in f:
                    if "MemFree:" in line:
                        free[path.split("/")[-2]] = round(int(line.split()[-2]) / 1e6, 1)   # kB -> GB
        out["node_free_gb"] = free
    except Exception:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from before
    the warm-up (so the tool's start-up overlaps no timed loop) until stop();
    the summary keeps the samples taken inside the marked timed windows."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device, interval_ms=50):
        self.device = device
        self.interval_ms = interval_ms
        self.samples = []   # (host time, fields)
        self.windows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.perf_counter(), [x.strip() for x in line.split(",")]))

    def mark(self, t0, t1):
        self.windows.append((t0, t1))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.proc = None

    def __enter__(self):
        return self.start()

    def __exit__(self, *a):
        self.stop()

    def summary(self):
        inside = [f for t, f in self.samples if any(a <= t <= b for a, b in self.windows)]
        rows = inside or [f for _, f in self.samples]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in rows if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in rows if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in rows for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "samples_from": "timed loops" if inside else "whole run (no sample inside a timed loop)"}


# ---------------------------------------------------------------------------
# workloads and the reference library

def spec_of(name):
    from fame_gb300 import synth
    return synth.WORKLOADS[name]


def chunk_list(rs, chunk):
    seq, offs = rs.concat()
    n = len(rs)
    out = []
    for c0 in range(0, n, chunk):
        c1 = min(n, c0 + chunk)
        o = offs[c0:c1 + 1].copy()
        out.append((int(o[0]), o - o[0]))
    return np.frombuffer(seq, np.uint8), out


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ref_library(readlen, maxpdist=550, build_if_missing=False):
    """(RefLib of the reference compiled with these constants, None) or (None, why)."""
    try:
        from oracle import refbind
        if not refbind.available(readlen, maxpdist) and build_if_missing:
            import __graft_entry__
            __graft_entry__.build()
        if not refbind.available(readlen, maxpdist):
            return None, "reference not built for READLEN %d / MAXPDIST %d (oracle/build_ref.sh)" % (readlen, maxpdist)
        return refbind.RefLib(refbind.variant_path(readlen, maxpdist)), None
    except Exception as e:   # a library that fails to load
        return None, "reference library unavailable: %s" % e


def ref_index_from_host(L, hi):
    """The reference's RefGenome filled with the tables of an index built by
    fame_index_build (equal to the reference constructor's, tests/test_index_build.py)."""
    t = hi.tables(sparse=False)

    class Arrays:
        pass

    a = Arrays()
    a.chrom_seqs = hi.chrom_seqs()
    a.chrom_names = hi.chrom_names()
    for k, v in t.items():
        setattr(a, k, v)
    a.tab_index64 = hi.tab_index64
    ri = L.from_arrays(a)
    del a, t
    gc.collect()
    return ri


def compare_se(got, ref):
    """Per-read and per-CpG comparison of two single-end results."""
    bad_reads = int(((got["mat"] != ref["mat"]) | (got["invalid"] != ref["invalid"])).sum())
    bad_cpgs = int((got["meth"] != ref["meth"]).any(1).sum())
    return {"reads": int(len(got["mat"])), "mismatched_reads": bad_reads, "mismatched_cpgs": bad_cpgs,
            "counters_equal": bool(np.array_equal(np.asarray(got["counters"], np.uint64),
                                                  np.asarray(ref["counters"], np.uint64)))}


# ---------------------------------------------------------------------------
def fastq_file_leg(gm, rs, slots=3):
    """Whole-file form (fame_match_fastq): the workload's reads written as a
    plain FASTQ file, parsed by the native reader straight into queue slots
    while earlier chunks run, strand vote on chunk 0; host clock around the
    call.  The second of two calls is reported (the file is then in the page
    cache); each call opens and frees its own queue."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp(prefix="fame_bench_")
    try:
        path = os.path.join(d, "reads.fq")
        t0 = time.perf_counter()
        rs.write_fastq(path)
        t_write = time.perf_counter() - t0
        size = os.path.getsize(path)
        times = []
        for _ in range(2):
            t0 = time.perf_counter()
            cnt, n = gm.match_fastq(path, False, 0, slots=slots, threads=0)
            times.append(time.perf_counter() - t0)
        gm.tallies(reset=True)
        out = {"value": n / times[-1], "unit": "reads/s", "reads": n, "file_bytes": size,
               "first_call_reads_per_s": n / times[0], "write_seconds": t_write, "slots": slots,
               "matched": int(cnt.succ),
               "timing": "host clock around fame_match_fastq: parse + copy + match + tallies, file in page cache"}
        out["bgzf"] = bgzf_leg(gm, rs, d, slots)
        return out
    finally:
        shutil.rmtree(d, ignore_errors=True)


def bgzf_leg(gm, rs, d, slots, n_reads=3_000_000):
    """gzip input written as BGZF (the first n_reads reads, level 1): the
    same file read by the native reader with its members inflated on the GPU
    and with zlib on one host thread (read only), then matched whole through
    fame_match_fastq (inflate on the GPU, parse, match, tallies); host clock,
    file in the page cache, second of two calls."""
    from fame_gb300 import synth
    from fame_gb300._lib import FastqReader
    sub = synth.ReadSet(seqs=rs.seqs[:n_reads], lens=rs.lens[:n_reads], chrom=rs.chrom[:n_reads],
                        start=rs.start[:n_reads], fwd=rs.fwd[:n_reads]) if len(rs) > n_reads else rs
    plain, path = os.path.join(d, "sub.fq"), os.path.join(d, "sub.fq.gz")
    sub.write_fastq(plain)
    t0 = time.perf_counter()
    synth.bgzf_compress(plain, path, level=1)
    t_comp = time.perf_counter() - t0
    text = os.path.getsize(plain)
    os.remove(plain)

    def read_through(device):
        r = FastqReader(path, is_gz=True, n_threads=0, max_reads=300000, max_len=256, device=device)
        assert r.gpu_inflate == (device >= 0)
        n = 0
        t0 = time.perf_counter()
        while True:
            _, offs = r.read()
            k = len(offs) - 1
            n += k
            if k < 300000:
                break
        dt = time.perf_counter() - t0
        r.close()
        return n, dt

    read_through(0)
    n_g, t_g = read_through(0)
    n_z, t_z = read_through(-1)
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        cnt, n = gm.match_fastq(path, True, 0, slots=slots, threads=0)
        times.append(time.perf_counter() - t0)
    gm.tallies(reset=True)
    return {"value": n / times[-1], "unit": "reads/s", "reads": n, "file_bytes": os.path.getsize(path),
            "text_bytes": text, "compress_seconds": t_comp, "matched": int(cnt.succ),
            "read_gpu_inflate": {"reads_per_s": n_g / t_g, "text_gb_per_s": text / t_g / 1e9},
            "read_zlib_one_thread": {"reads_per_s": n_z / t_z, "text_gb_per_s": text / t_z / 1e9},
            "timing": "host clock: reader alone (inflate + parse) both ways, then fame_match_fastq on the BGZF file "
                      "(GPU inflate, parse, copy, match, tallies)"}


def run_gb300(args):
    import torch
    from fame_gb300 import (CHUNKSIZE, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, GpuQueue, HostIndex,
                            synth)
    from fame_gb300._lib import lib as _L
    rank, world, local = dist_init(args.gpus)
    t0 = time.time()
    g = synth.genome_of(args.workload)
    rs, readlen = synth.reads_of(args.workload, g, args.reads)
    t_gen = time.time() - t0
    hi, t_build, index_rep = build_index(args, g.seqs, readlen, local)
    genome_bp, n_chrom = int(g.total_len), len(g.seqs)
    del g
    gc.collect()
    t0 = time.time()
    gm = GpuMatcher(hi, local)
    t_open = time.time() - t0
    seq, chunks = chunk_list(rs, CHUNKSIZE)
    # chunk 0 runs the strand vote in the warm-up; the timed steps cycle over this rank's later chunks
    mine = [i for i in range(len(chunks)) if i % world == rank] or [0]
    first = mine[0]
    steady = [i for i in mine if i != 0] or mine
    used = sorted({first} | set(steady[:max(args.steps, args.warmup, 1)]))
    dev, pinned = {}, {}
    maxn = max(len(chunks[i][1]) - 1 for i in used)
    d_mat = gm.alloc(8 * maxn)
    d_inv = gm.alloc(maxn)
    for i in used:
        # each chunk in page-locked host memory, and the device copy filled from
        # there (so every host buffer has served a copy before the timed loops,
        # as a host's reused staging buffers have)
        base, o = chunks[i]
        nb = int(o[-1])
        hs = gm.host_alloc(nb)
        ho = gm.host_alloc(8 * len(o)).view(np.uint64)
        hs[:] = seq[base:base + nb]
        ho[:] = o
        pinned[i] = (hs, ho, len(o) - 1)
        d_s = gm.alloc(nb)
        d_o = gm.alloc(8 * len(o))
        gm.memcpy(d_s, hs.ctypes.data, nb, 1)
        gm.memcpy(d_o, ho.ctypes.data, 8 * len(o), 1)
        dev[i] = (d_s, d_o, len(o) - 1)
    h_mat = gm.host_alloc(8 * maxn).view(np.uint64)
    h_inv = gm.host_alloc(maxn)
    # where the page-locked chunk buffers landed (a buffer off the GPU's near
    # node copies over the CPU-to-CPU link)
    near = gm.host_node()
    buf_nodes = {i: sorted(set(gm.page_nodes(pinned[i][0]) + gm.page_nodes(pinned[i][1]))) for i in used}
    p_stream = ctypes.c_void_p()
    _L().fame_gpu_stream(gm.h, ctypes.byref(p_stream))
    stream = torch.cuda.ExternalStream(p_stream.value, device=local)
    clk = ClockSampler(local).start()
    # warm-up: chunk 0 with the strand vote (getStranded), then the decided orientation
    d_s, d_o, n = dev[first]
    c = gm.match_reads_dev(d_s, d_o, n, FAME_GET_STRANDED, d_mat, d_inv)
    flags = FAME_MATCH_R1_FWD if c.r1_fwd > c.r1_rev else 0
    for w in range(max(0, args.warmup - 1)):
        d_s, d_o, n = dev[steady[w % len(steady)]]
        gm.match_reads_dev(d_s, d_o, n, flags, d_mat, d_inv)
    gm.set_timing(True)
    # ---- timed: plain form, reads resident in HBM
    stage = np.zeros(len(GpuMatcher.STAGES))
    tiers = np.zeros(5)
    reads = gather = scans = launches = heavy = reruns = dp = inv_len = succ = 0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    ev0.record(stream)
    tw0 = time.perf_counter()
    host_steps = {"plain": [], "e2e": []}
    for k in range(args.steps):
        d_s, d_o, n = dev[steady[k % len(steady)]]
        th = time.perf_counter()
        c = gm.match_reads_dev(d_s, d_o, n, flags, d_mat, d_inv)
        host_steps["plain"].append(time.perf_counter() - th)
        stage += gm.stage_times()
        tiers += gm.seed_tier_counts()
        reads += n
        gather += c.gather_bytes
        scans += c.windows_scanned
        heavy += c.heavy_tasks
        reruns += c.reruns
        dp += c.dp_reads
        inv_len += c.invalid_len
        succ += c.succ
        launches += gm.last_launches()
    ev1.record(stream)
    torch.cuda.synchronize()
    tw1 = time.perf_counter()
    clk.mark(tw0, tw1)
    barrier(world)
    t_max = allreduce_max(ev0.elapsed_time(ev1) / 1e3, world)
    total_reads = reads * world
    # ---- host-to-device copy rate of one chunk's page-locked bases (synchronous copies, host clock)
    hs0, _, _ = pinned[steady[0]]
    d_s0 = dev[steady[0]][0]
    gm.memcpy(d_s0, hs0.ctypes.data, hs0.nbytes, 1)
    tc0 = time.perf_counter()
    for _ in range(3):
        gm.memcpy(d_s0, hs0.ctypes.data, hs0.nbytes, 1)
    h2d_gbps = 3 * hs0.nbytes / (time.perf_counter() - tc0) / 1e9
    # ---- timed: end to end from page-locked host memory
    e_reads = h2d = d2h = 0
    e2e_steps = []
    for w in range(args.warmup):   # untimed: the host-buffer path's first calls (its device staging grows)
        hs, ho, n = pinned[steady[w % len(steady)]]
        gm.match_reads(hs, ho, flags, mats=h_mat[:n], invalid=h_inv[:n])
    barrier(world)
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    ev0.record(stream)
    for k in range(args.steps):
        hs, ho, n = pinned[steady[k % len(steady)]]
        th = time.perf_counter()
        gm.match_reads(hs, ho, flags, mats=h_mat[:n], invalid=h_inv[:n])
        host_steps["e2e"].append(time.perf_counter() - th)
        e2e_steps.append((steady[k % len(steady)], time.perf_counter() - th))
        e_reads += n
        h2d += hs.nbytes + ho.nbytes
        d2h += 9 * n
    ev1.record(stream)
    torch.cuda.synchronize()
    clk.mark(te0, time.perf_counter())
    t_e2e = allreduce_max(ev0.elapsed_time(ev1) / 1e3, world)
    gm.set_timing(False)
    # ---- batched form: launch shapes autotuned on the first steady chunk
    # (fame_gpu_autotune: seeding tiers, window-scan and DP grids; it checks
    # that every shape gives the same results), then the same steps through
    # the queue (CUDA-graph chunk slots on their own streams, persistent
    # seeding and scan kernels taking work from device queues, the copies of
    # one chunk overlapping the kernels of another), from the same host
    # buffers; host clock between two device synchronisations (the work spans
    # several streams)
    import tempfile
    tune_path = os.path.join(tempfile.gettempdir(), "fame_tuning_%d.json" % os.getpid())
    t0 = time.time()
    d_s, d_o, n = dev[steady[0]]
    tuning = gm.autotune(d_s, d_o, n, flags, tune_path)
    t_tune = time.time() - t0
    nslots = 3
    q = GpuQueue(gm, nslots, maxn, max(int(p[0].nbytes) for p in pinned.values()))
    for w in range(nslots):
        hs, ho, n = pinned[steady[w % len(steady)]]
        q.collect(q.submit(hs, ho, flags))
    launches_q0 = q.launches()
    b_reads = 0
    inflight = []
    barrier(world)
    torch.cuda.synchronize()
    tb0 = time.perf_counter()
    for k in range(args.steps):
        if len(inflight) == nslots:
            s_, n_ = inflight.pop(0)
            q.collect(s_, mats=h_mat[:n_], invalid=h_inv[:n_])
        hs, ho, n = pinned[steady[k % len(steady)]]
        inflight.append((q.submit(hs, ho, flags), n))
        b_reads += n
    for s_, n_ in inflight:
        q.collect(s_, mats=h_mat[:n_], invalid=h_inv[:n_])
    torch.cuda.synchronize()
    tb1 = time.perf_counter()
    clk.mark(tb0, tb1)
    clk.stop()
    t_b = allreduce_max(tb1 - tb0, world)
    batched = {"value": b_reads * world / t_b, "unit": "reads/s", "slots": nslots,
               "vs_plain": (b_reads * world / t_b) / (total_reads / t_max),
               "gpu_launches": q.launches() - launches_q0,
               "tuning": {k: tuning[k] for k in ("seed_mode", "sa_blocks_per_sm", "dp_blocks_per_sm")},
               "tuning_seconds": t_tune,
               "tuning_trials": [[t["seed_mode"], t["sa_blocks_per_sm"], t["dp_blocks_per_sm"],
                                  round(t["stage_ms"][1] + t["stage_ms"][5], 3), round(t["stage_ms"][2], 3),
                                  round(t["stage_ms"][4], 3)] for t in tuning["trials"]],
               "tuning_trials_columns": ["seed_mode", "sa_blocks_per_sm", "dp_blocks_per_sm", "seed_ms",
                                         "shift_and_ms", "dp_ms"],
               "timing": "host clock between device synchronisations; host buffers in and out"}
    q.close()
    fastq = fastq_file_leg(gm, rs) if (rank == 0 and not args.no_fastq) else None
    # ---- parity sample: the first reads of chunk 1 in the decided orientation
    # on the GPU (tallies of the sample alone), checked below against the reference
    sample = None
    if rank == 0 and not args.no_cpu_baseline:
        sc = 1 if len(chunks) > 1 else 0
        base, o = chunks[sc]
        ns = min(args.cpu_sample, len(o) - 1)
        so = o[:ns + 1].copy()
        ss = seq[base:base + int(so[-1])].tobytes()
        gm.tallies(reset=True)
        m, iv, cc = gm.match_reads(ss, so, flags)
        sample = dict(seq=ss, offs=so, chunk=sc,
                      got=dict(mat=m, invalid=iv, meth=gm.tallies(reset=True),
                               counters=[cc.succ, cc.nonunique, cc.unsucc]))
    # ---- roofline of the index-gather kernel
    hbm, src = peaks()
    names = ["read_prep", "seed_gather", "shift_and", "select_exact_cpg", "banded_dp", "seed_heavy",
             "seed_mid_small", "seed_mid_large", "seed_global"]
    st = {names[i]: stage[i] / 1e3 for i in range(len(names))}
    dominant = max(names[:6], key=lambda k: st[k])
    seed_s = st["seed_gather"] + st["seed_heavy"]
    gbps = gather / seed_s / 1e9 if seed_s > 0 else 0.0
    fig = NCU_FIGURES.get(args.workload) if not args.reads else None
    src_hash = kernel_source_hash()
    fig_ok = bool(fig) and fig.get("source_hash") == src_hash
    traffic = fig["seed_traffic_per_step"] if fig_ok else None
    out = {
        "metric": METRIC, "value": total_reads / t_max, "unit": "reads/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 integer",
        "data": "synthetic (seeded genome and bisulfite reads per the workload definition, fame_gb300/synth.py)",
        "config": {"workload": args.workload, "genome_bp": genome_bp, "chromosomes": n_chrom,
                   "reads_total": len(rs), "read_len": readlen,
                   "read_lengths": [int(rs.lens.min()), int(rs.lens.max())], "chunk_reads": CHUNKSIZE,
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2: every step gathers from the device index (%.1f GB) and new reads"
                         % (gm.index_bytes() / 1e9)},
        "e2e": {"value": e_reads * world / t_e2e, "unit": "reads/s", "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": int(d2h / args.steps), "h2d_copy_gbps": h2d_gbps},
        "gpu_launches": launches,
        "host_step_ms": {k: [round(1e3 * min(v), 3), round(1e3 * float(np.median(v)), 3), round(1e3 * max(v), 3)]
                         for k, v in host_steps.items() if v},
        "batched": batched,
        "fastq_file": fastq,
        "stage_seconds": st,
        "dominant_kernel": dominant,
        "counts": {"reads": reads, "matched": succ, "invalid_len": inv_len, "dp_reads": dp,
                   "windows_scanned_per_read": scans / max(1, reads), "heavy_seed_tasks": heavy,
                   "seed_tier_tasks": {"mid_small": int(tiers[0]), "mid_large": int(tiers[1]),
                                       "global": int(tiers[2]), "large_capacity": int(tiers[3]),
                                       "replayed_orders": int(tiers[4])},
                   "candidate_overflow_reruns": reruns},
        "roofline": {"kernel": "seeding (k_seed_mid and the other seeding tiers: index gathers)", "bound": "hbm", "achieved": gbps, "peak": hbm,
                     "unit": "GB/s", "frac": gbps / hbm, "traffic": traffic,
                     "dram_achieved": traffic / (seed_s / args.steps) / 1e9 if (traffic and seed_s > 0) else None,
                     "note": "algorithmic bytes = 8 B bucket bounds + 4 B per bucket entry per k-mer lookup, "
                             "counted on the device; peak %s; traffic = DRAM read + write of the seeding launches "
                             "of one steady-state chunk from ncu (%s)" % (src, fig["profile"] if fig_ok else
                                                       "no capture of the current kernel sources")},
        "alu_bound_kernels": {
            "k_shiftand": {"stage_ms": 1e3 * st["shift_and"] / args.steps,
                           "alu_pipe_of_peak": fig.get("shiftand_alu") if fig_ok else None},
            "k_dp_warp": {"stage_ms": 1e3 * st["banded_dp"] / args.steps,
                          "alu_pipe_of_peak": fig.get("dp_alu") if fig_ok else None},
            "note": "stages bound by the integer/logic pipe, not by HBM or tensor cores; ALU-pipe figures from "
                    "ncu captures of the same kernel sources (kernel source hash %s)" % src_hash},
        "host": dict(host_placement(local), near_node=near,
                     e2e_steps=[{"chunk": c, "ms": round(1e3 * t, 3), "buffer_nodes": buf_nodes.get(c)}
                                for c, t in e2e_steps],
                     off_node_chunk_buffers=sum(1 for v in buf_nodes.values() if near >= 0 and any(x != near for x in v)),
                     chunk_buffers=len(buf_nodes)),
        "clocks": clk.summary(),
        "setup_seconds": {"generate": t_gen, "index_build": t_build, "upload": t_open},
        "index_build": index_rep,
    }
    for i in used:
        gm.free(dev[i][0])
        gm.free(dev[i][1])
    gm.close()
    del dev, pinned, h_mat, h_inv
    gc.collect()
    if sample is not None:
        out["cpu_baseline"], out["parity"] = cpu_baseline_se(hi, readlen, sample, flags)
    if rank == 0:
        emit(out)


def cpu_baseline_se(hi, readlen, sample, flags):
    """The reference's OpenMP matchReads on the sample (decided orientation, the
    steady state), timed; its per-read results and tallies compared with the GPU's."""
    from fame_gb300 import FAME_MATCH_R1_FWD
    L, why = ref_library(readlen)
    n = len(sample["offs"]) - 1
    if L is None:
        return {"value": None, "unit": "reads/s", "cores": 0, "kind": "reference", "sample": why}, \
            {"reads": n, "checked": False, "why": why}
    t0 = time.time()
    ri = ref_index_from_host(L, hi)
    t_load = time.time() - t0
    secs, cnt, ref = ri.time_se(sample["seq"], sample["offs"], both_strands=False,
                                match_r1_fwd=bool(flags & FAME_MATCH_R1_FWD), outputs=True)
    ri.close()
    ref["counters"] = [int(x) for x in cnt[:3]]
    par = compare_se(sample["got"], ref)
    par.update(checker="reference (oracle/_ref, its matchReads on the same index tables)", chunk=sample["chunk"])
    base = {"value": n / secs, "unit": "reads/s", "cores": L.corenum, "kind": "reference",
            "sample": "%d reads of chunk %d (300k-read CHUNKSIZE), decided orientation, matchReads only, "
                      "CORENUM=%d OpenMP threads, READLEN %d" % (n, sample["chunk"], L.corenum, L.readlen),
            "seconds": secs, "index_load_seconds": t_load}
    return base, par


# ---------------------------------------------------------------------------
SERVING_METRIC = "aggregate reads/s of a single-cell job stream (serving form), with p50/p99 job latency"


def run_gb300_serving(args):
    """Serving form: single-cell jobs arrive as a Poisson stream; the serving
    loop (fame_gb300/serving.py) admits them into the batched queue while
    others run; the plain per-job path runs the same trace job after job."""
    from fame_gb300 import GpuMatcher, HostIndex, synth
    from fame_gb300.serving import Job, ServingLoop, latency_summary, plain_per_job
    spec = synth.WORKLOADS[args.workload]
    js = spec["jobs"]
    rng = np.random.default_rng(js["seed"])
    sizes = np.clip(np.round(js["median"] * np.exp(js["sigma"] * rng.standard_normal(js["n_jobs"]))),
                    js["lo"], js["hi"]).astype(np.int64)
    arrivals = np.cumsum(rng.exponential(1.0 / js["rate"], js["n_jobs"]))
    t0 = time.time()
    jobs = []
    cell_p = None
    if spec.get("large"):
        # genome-scale genome; every cell its own methylation probability (Beta) and its own reads
        g = synth.genome_of(args.workload)
        cell_p = rng.beta(*js["cell_beta"], size=js["n_jobs"])
        for i, n in enumerate(sizes):
            rs = synth.make_reads_large(g, int(n), seed=js["seed"] + 1 + i, read_len=100, sub_rate=js["sub_rate"],
                                        indel_rate=js["indel_rate"], cell_p=float(cell_p[i]), cell_key=i)
            s_, o_ = rs.concat()
            jobs.append(Job("cell%d" % i, s_, o_, arrival=float(arrivals[i])))
    else:
        g = synth.make_genome(**spec["genome"])
        rs = synth.make_reads(g, int(sizes.sum()), seed=js["seed"] + 1, sub_rate=js["sub_rate"],
                              indel_rate=js["indel_rate"])
        seq, offs = rs.concat()
        a = 0
        for i, n in enumerate(sizes):
            o = offs[a:a + n + 1]
            jobs.append(Job("cell%d" % i, seq[int(o[0]):int(o[-1])], o - o[0], arrival=float(arrivals[i])))
            a += int(n)
    t_gen = time.time() - t0
    hi, t_build, index_rep = build_index(args, g.seqs, 100, 0)
    genome_bp = int(g.total_len)
    del g
    gc.collect()
    gm = GpuMatcher(hi, 0)
    loop = ServingLoop(gm, slots=4, max_active=16)
    loop.run(jobs[:2], realtime=False)                       # warm-up (graphs, buffers)
    plain_per_job(gm, jobs[:1], realtime=False)
    with ClockSampler(0) as clk:
        t1 = time.perf_counter()
        served = loop.run(jobs, realtime=True)
        t_serv = time.perf_counter() - t1
        clk.mark(t1, t1 + t_serv)
        t1 = time.perf_counter()
        plain = plain_per_job(gm, jobs, realtime=True)
        t_plain = time.perf_counter() - t1
    same = all(np.array_equal(a.meth, b.meth) and a.counters == b.counters
               for a, b in zip(sorted(served, key=lambda r: r.job_id), sorted(plain, key=lambda r: r.job_id)))
    loop.close()
    gm.close()
    total = int(sizes.sum())
    out = {
        "metric": SERVING_METRIC, "value": total / t_serv, "unit": "reads/s", "n_gpus": 1, "steps": 1,
        "warmup": 1, "ms_per_step": 1e3 * t_serv, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u64 integer", "data": "synthetic (seeded jobs and arrival trace)",
        "config": {"workload": args.workload, "genome_bp": genome_bp, "jobs": len(jobs), "reads_total": total,
                   "arrival_rate_per_s": js["rate"], "reads_per_job_median": js["median"],
                   "reads_per_job_range": [int(sizes.min()), int(sizes.max())], "slots": 4,
                   "cell_methylation_p": (None if cell_p is None else
                                          {"beta": list(js["cell_beta"]),
                                           "range": [float(cell_p.min()), float(cell_p.max())]})},
        "latency": {"serving": latency_summary(served), "plain_per_job": latency_summary(plain)},
        "plain_per_job_reads_per_s": total / t_plain,
        "results_identical_to_plain": bool(same),
        "timing": "host clock over the whole trace (arrival-driven); per-job latency = completion - arrival",
        "clocks": clk.summary(), "setup_seconds": {"generate": t_gen, "index_build": t_build},
        "index_build": index_rep,
    }
    emit(out)


# ---------------------------------------------------------------------------
def run_gb300_pe(args):
    """Paired-end form: one step = one 300k-pair chunk through matchPairedReads
    semantics (fame_gpu_match_pairs_dev; mates resident in HBM), e2e through
    fame_gpu_match_pairs from page-locked host buffers."""
    import torch
    from fame_gb300 import CHUNKSIZE, FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, HostIndex, synth
    from fame_gb300._lib import lib as _L
    spec = spec_of(args.workload)
    maxpdist = int(spec.get("maxpdist", 550))
    t0 = time.time()
    g = synth.genome_of(args.workload)
    r1, r2 = synth.pairs_of(args.workload, g, args.reads)
    t_gen = time.time() - t0
    hi, t_build, index_rep = build_index(args, g.seqs, 100, 0)
    genome_bp = int(g.total_len)
    del g
    gc.collect()
    t0 = time.time()
    gm = GpuMatcher(hi, 0)
    t_open = time.time() - t0
    s1, o1 = r1.concat()
    s2, o2 = r2.concat()
    n = len(o1) - 1
    chunks = [(c0, min(n, c0 + CHUNKSIZE)) for c0 in range(0, n, CHUNKSIZE)]
    steady = list(range(1, len(chunks))) or [0]
    used = sorted({0} | set(steady[:max(args.steps, args.warmup, 1)]))
    dev, pinned = {}, {}
    maxn = max(chunks[i][1] - chunks[i][0] for i in used)
    d_mat = gm.alloc(16 * maxn)
    d_inv = gm.alloc(2 * maxn)
    b1a, b2a = np.frombuffer(s1, np.uint8), np.frombuffer(s2, np.uint8)
    for i in used:
        a, b = chunks[i]
        m1 = b1a[int(o1[a]):int(o1[b])]
        m2 = b2a[int(o2[a]):int(o2[b])]
        oo = np.concatenate([o1[a:b + 1] - o1[a], (o2[a + 1:b + 1] - o2[a]) + (o1[b] - o1[a])]).astype(np.uint64)
        h1 = gm.host_alloc(len(m1)); h1[:] = m1
        h2 = gm.host_alloc(len(m2)); h2[:] = m2
        ho1 = gm.host_alloc(8 * (b - a + 1)).view(np.uint64); ho1[:] = o1[a:b + 1] - o1[a]
        ho2 = gm.host_alloc(8 * (b - a + 1)).view(np.uint64); ho2[:] = o2[a:b + 1] - o2[a]
        pinned[i] = (h1, ho1, h2, ho2, b - a)
        # the device copy (mates back to back) filled from the page-locked buffers, so
        # that each has served a copy before the timed loops
        d_s = gm.alloc(len(m1) + len(m2))
        d_o = gm.alloc(8 * len(oo))
        gm.memcpy(d_s, h1.ctypes.data, len(m1), 1)
        gm.memcpy(d_s + len(m1), h2.ctypes.data, len(m2), 1)
        gm.memcpy(d_o, ho1.ctypes.data, ho1.nbytes, 1)
        gm.memcpy(d_o, ho2.ctypes.data, ho2.nbytes, 1)
        gm.memcpy(d_o, oo.ctypes.data, 8 * len(oo), 1)
        dev[i] = (d_s, d_o, b - a)
    p_stream = ctypes.c_void_p()
    _L().fame_gpu_stream(gm.h, ctypes.byref(p_stream))
    stream = torch.cuda.ExternalStream(p_stream.value, device=0)
    clk = ClockSampler(0).start()
    d_s, d_o, nn = dev[0]
    c = gm.match_pairs_dev(d_s, d_o, nn, FAME_GET_STRANDED, maxpdist, d_mat, d_inv)
    flags = FAME_MATCH_R1_FWD if c.r1_fwd > c.r1_rev else 0
    for w in range(max(0, args.warmup - 1)):
        d_s, d_o, nn = dev[steady[w % len(steady)]]
        gm.match_pairs_dev(d_s, d_o, nn, flags, maxpdist, d_mat, d_inv)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pairs = launches = heavy = paired = 0
    # per-stage CUDA-event times, from one extra untimed chunk
    gm.set_timing(True)
    d_s, d_o, nn = dev[steady[0]]
    gm.match_pairs_dev(d_s, d_o, nn, flags, maxpdist, d_mat, d_inv)
    pe_stages = {k: float(v) for k, v in zip(GpuMatcher.PAIR_STAGES, gm.pair_stage_times())}
    gm.set_timing(False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    for k in range(args.steps):
        d_s, d_o, nn = dev[steady[k % len(steady)]]
        c = gm.match_pairs_dev(d_s, d_o, nn, flags, maxpdist, d_mat, d_inv)
        pairs += nn
        heavy += c.heavy_pairs
        paired += c.paired
        launches += gm.last_launches()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk.mark(t0, time.perf_counter())
    t_dev = ev0.elapsed_time(ev1) / 1e3
    for w in range(args.warmup):
        h1, ho1, h2, ho2, nn = pinned[steady[w % len(steady)]]
        gm.match_pairs(h1, ho1, h2, ho2, flags, maxpdist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    e_pairs = h2d = d2h = 0
    for k in range(args.steps):
        h1, ho1, h2, ho2, nn = pinned[steady[k % len(steady)]]
        gm.match_pairs(h1, ho1, h2, ho2, flags, maxpdist)
        e_pairs += nn
        h2d += h1.nbytes + h2.nbytes + 16 * (nn + 1)
        d2h += 18 * nn
    ev1.record(stream)
    torch.cuda.synchronize()
    clk.mark(t0, time.perf_counter())
    clk.stop()
    t_e2e = ev0.elapsed_time(ev1) / 1e3
    # parity sample: the first pairs of chunk 1 in the decided orientation
    sample = None
    if not args.no_cpu_baseline:
        sc = 1 if len(chunks) > 1 else 0
        c0, c1 = chunks[sc]
        ns = min(args.cpu_sample, c1 - c0)
        p1 = o1[c0:c0 + ns + 1]
        p2 = o2[c0:c0 + ns + 1]
        q1, q2 = s1[int(p1[0]):int(p1[-1])], s2[int(p2[0]):int(p2[-1])]
        gm.tallies(reset=True)
        m1, m2, i1, i2, cc = gm.match_pairs(q1, p1 - p1[0], q2, p2 - p2[0], flags, maxpdist)
        sample = dict(s1=q1, o1=p1 - p1[0], s2=q2, o2=p2 - p2[0], chunk=sc,
                      got=dict(mat1=m1, mat2=m2, inv1=i1, inv2=i2, meth=gm.tallies(reset=True),
                               counters=[cc.succ, cc.nonunique, cc.unsucc, cc.paired, cc.too_short]))
    out = {
        "metric": PE_METRIC, "value": pairs / t_dev, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 integer",
        "data": "synthetic (seeded genome and bisulfite read pairs per the workload definition)",
        "config": {"workload": args.workload, "genome_bp": genome_bp, "pairs_total": n, "read_len": 100,
                   "chunk_pairs": CHUNKSIZE, "maxpdist": maxpdist, "parallelism": "single GPU",
                   "l2": "inputs larger than L2: every step gathers from the device index (%.1f GB) and new pairs"
                         % (gm.index_bytes() / 1e9)},
        "e2e": {"value": e_pairs / t_e2e, "unit": "pairs/s", "h2d_bytes_per_step": int(h2d / args.steps),
                "d2h_bytes_per_step": int(d2h / args.steps)},
        "gpu_launches": launches, "counts": {"pairs": pairs, "paired": paired, "heavy_pairs": heavy},
        "stage_ms_one_chunk": pe_stages,
        "clocks": clk.summary(),
        "setup_seconds": {"generate": t_gen, "index_build": t_build, "upload": t_open},
        "index_build": index_rep,
    }
    for d_s, d_o, _ in dev.values():
        gm.free(d_s)
        gm.free(d_o)
    gm.close()
    del dev, pinned
    gc.collect()
    if sample is not None:
        out["cpu_baseline"], out["parity"] = cpu_baseline_pe(hi, maxpdist, sample, flags)
    emit(out)


def cpu_baseline_pe(hi, maxpdist, sample, flags):
    """The reference's OpenMP matchPairedReads on the sample, timed; per-mate
    results and tallies compared with the GPU's."""
    from fame_gb300 import FAME_MATCH_R1_FWD
    L, why = ref_library(100, maxpdist)
    n = len(sample["o1"]) - 1
    if L is None:
        return {"value": None, "unit": "pairs/s", "cores": 0, "kind": "reference", "sample": why}, \
            {"pairs": n, "checked": False, "why": why}
    ri = ref_index_from_host(L, hi)
    secs, cnt, ref = ri.time_pe(sample["s1"], sample["o1"], sample["s2"], sample["o2"], both_strands=False,
                                match_r1_fwd=bool(flags & FAME_MATCH_R1_FWD), outputs=True)
    ri.close()
    got = sample["got"]
    bad = int(((got["mat1"] != ref["mat1"]) | (got["mat2"] != ref["mat2"]) | (got["inv1"] != ref["inv1"]) |
               (got["inv2"] != ref["inv2"])).sum())
    par = {"pairs": n, "mismatched_pairs": bad, "mismatched_cpgs": int((got["meth"] != ref["meth"]).any(1).sum()),
           "counters_equal": bool(np.array_equal(np.asarray(got["counters"], np.uint64), cnt[:5])),
           "checker": "reference (oracle/_ref, its matchPairedReads on the same index tables)",
           "chunk": sample["chunk"]}
    base = {"value": n / secs, "unit": "pairs/s", "cores": L.corenum, "kind": "reference",
            "sample": "%d pairs of chunk %d, decided orientation, matchPairedReads only, CORENUM=%d OpenMP "
                      "threads, MAXPDIST %d" % (n, sample["chunk"], L.corenum, L.maxpdist()), "seconds": secs}
    return base, par


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference's own OpenMP matching on the machine's host cores, on bounded
    samples of the same chunks (decided orientation).  Its index: the
    reference's own constructor for the 300 Mbp workloads; for the 3 Gbp ones
    (about 70 minutes in that constructor) the tables fame_index_build
    produces, loaded into the reference's RefGenome (the same tables)."""
    rank, world, local = dist_init(args.gpus)
    if rank != 0:
        return
    from fame_gb300 import CHUNKSIZE, HostIndex, synth
    spec = spec_of(args.workload)
    paired = "pairs" in spec
    readlen = 100 if paired else int(spec["reads"].get("read_len", 100))
    maxpdist = int(spec.get("maxpdist", 550)) if paired else 550
    L, why = ref_library(readlen, maxpdist, build_if_missing=True)
    if L is None:
        emit({"impl": "reference", "unavailable": why})
        return
    g = synth.genome_of(args.workload)
    if paired:
        r1, r2 = synth.pairs_of(args.workload, g, args.reads)
    else:
        rs, _ = synth.reads_of(args.workload, g, args.reads)
    t0 = time.time()
    if spec.get("large"):
        hi = HostIndex.build(g.seqs, readlen=readlen, threads=0)
        del g
        gc.collect()
        ri = ref_index_from_host(L, hi)
        hi.close()
        how = "tables of fame_index_build loaded into the reference's RefGenome"
    else:
        fasta = "/tmp/fame_bench_%s.fa" % args.workload
        g.write_fasta(fasta)
        ri = L.build(fasta)   # the reference's own readReference + RefGenome constructor
        how = "the reference's own constructor"
    t_index = time.time() - t0
    sample = min(args.cpu_sample, CHUNKSIZE)
    if paired:
        s1, o1 = r1.concat()
        s2, o2 = r2.concat()
        n = len(o1) - 1
        starts = list(range(CHUNKSIZE, n, CHUNKSIZE)) or [0]

        def step(k):
            c0 = starts[k % len(starts)]
            nn = min(sample, n - c0)
            p1 = o1[c0:c0 + nn + 1]
            p2 = o2[c0:c0 + nn + 1]
            secs, _ = ri.time_pe(s1[int(p1[0]):int(p1[-1])], p1 - p1[0], s2[int(p2[0]):int(p2[-1])], p2 - p2[0],
                                 both_strands=False, match_r1_fwd=True)
            return secs, nn
        metric, unit = PE_METRIC, "pairs/s"
    else:
        seq, chunks = chunk_list(rs, CHUNKSIZE)
        steady = list(range(1, len(chunks))) or [0]

        def step(k):
            base, o = chunks[steady[k % len(steady)]]
            o = o[:sample + 1]
            secs, _ = ri.time_se(seq[base:base + int(o[-1])].tobytes(), o, both_strands=False, match_r1_fwd=True)
            return secs, len(o) - 1
        metric, unit = METRIC, "reads/s"
    for k in range(args.warmup):
        step(k)
    secs = 0.0
    units = 0
    for k in range(args.steps):
        s_, n_ = step(k)
        secs += s_
        units += n_
    v = units / secs
    emit({
        "impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8/u64 integer",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "per_step": sample, "read_len": readlen,
                   "maxpdist": maxpdist if paired else None},
        "cpu_baseline": {"value": v, "unit": unit, "cores": L.corenum, "kind": "reference",
                         "sample": "%d %s per step from consecutive 300k chunks, decided orientation; index: %s"
                                   % (sample, "pairs" if paired else "reads", how)},
        "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_seconds": {"index": t_index, "index_cores": L.corenum}})
    ri.close()


if __name__ == "__main__":
    stdout_to_stderr()
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif "pairs" in spec_of(a.workload):
        run_gb300_pe(a)
    elif "jobs" in spec_of(a.workload):
        run_gb300_serving(a)
    else:
        run_gb300(a)
