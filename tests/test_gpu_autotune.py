"""The launch-shape autotuner (fame_gpu_autotune / fame_gpu_load_tuning):
every shape it tries gives the same per-read results (it checks that itself),
the chosen shapes are written as JSON and loaded back, and the plain calls
and the queue give bit-identical results and tallies under the chosen
shapes."""
import json

import numpy as np
import pytest

from fame_gb300 import FAME_GET_STRANDED, FAME_MATCH_R1_FWD, GpuMatcher, GpuQueue, HostIndex, synth

pytestmark = pytest.mark.gpu


def test_autotune_keeps_results(tmp_path):
    g = synth.make_genome([300_000, 200_000], seed=71, repeat_frac=0.3, n_families=10, fam_len=(300, 2000),
                          divergence=(0.0, 0.05))
    rs = synth.make_reads(g, 30_000, seed=72, sub_rate=0.01, indel_rate=0.002, repeat_read_frac=0.2)
    seq, offs = rs.concat()
    n = len(offs) - 1
    hi = HostIndex.build(g.seqs, readlen=100)
    gm = GpuMatcher(hi, 0)
    path = str(tmp_path / "tuning.json")
    try:
        gm.tallies(reset=True)
        m0, i0, c0 = gm.match_reads(seq, offs, FAME_MATCH_R1_FWD)
        t0 = gm.tallies(reset=True)
        raw = np.frombuffer(seq, np.uint8)
        d_s, d_o = gm.alloc(len(raw)), gm.alloc(8 * (n + 1))
        gm.memcpy(d_s, raw.ctypes.data, len(raw), 1)
        gm.memcpy(d_o, offs.ctypes.data, 8 * (n + 1), 1)
        q = GpuQueue(gm, 2, n, len(raw))
        m2, i2, _ = q.collect(q.submit(seq, offs, FAME_MATCH_R1_FWD))   # a graph captured before tuning
        assert np.array_equal(m0, m2) and np.array_equal(i0, i2)
        assert np.array_equal(gm.tallies(reset=True), t0)
        choice = gm.autotune(d_s, d_o, n, FAME_MATCH_R1_FWD, path)
        assert {"seed_mode", "sa_blocks_per_sm", "dp_blocks_per_sm"} <= set(choice)
        assert len(choice["trials"]) == 4 + 3 + 2
        assert all(len(t["stage_ms"]) == len(GpuMatcher.STAGES) for t in choice["trials"])
        assert gm.seed_tier() == choice["seed_mode"]
        # the tuning run left the tallies alone; results under the chosen shapes are the same
        assert not gm.tallies().any()
        m1, i1, c1 = gm.match_reads(seq, offs, FAME_MATCH_R1_FWD)
        assert np.array_equal(m0, m1) and np.array_equal(i0, i1) and c0.succ == c1.succ
        assert np.array_equal(gm.tallies(reset=True), t0)
        m2, i2, _ = q.collect(q.submit(seq, offs, FAME_MATCH_R1_FWD))   # captured again with the new shapes
        q.close()
        assert np.array_equal(m0, m2) and np.array_equal(i0, i2)
        assert np.array_equal(gm.tallies(reset=True), t0)
        gm.free(d_s)
        gm.free(d_o)
    finally:
        gm.close()
    # loading the file on a new context applies the same shapes
    gm2 = GpuMatcher(hi, 0)
    try:
        gm2.load_tuning(path)
        assert gm2.seed_tier() == choice["seed_mode"]
        m3, i3, _ = gm2.match_reads(seq, offs, FAME_GET_STRANDED)
        m4, i4, _ = gm2.match_reads(seq, offs, FAME_GET_STRANDED)
        assert np.array_equal(m3, m4) and np.array_equal(i3, i4)
        bad = tmp_path / "bad.json"
        bad.write_text(json.dumps({"seed_mode": 9, "sa_blocks_per_sm": 8, "dp_blocks_per_sm": 2}))
        with pytest.raises(Exception):
            gm2.load_tuning(str(bad))
        with pytest.raises(Exception):
            gm2.load_tuning(str(tmp_path / "missing.json"))
        assert gm2.seed_tier() == choice["seed_mode"]   # a refused file changes nothing
    finally:
        gm2.close()
