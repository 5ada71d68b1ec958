"""Read-sharded matching across 2 processes (gloo on CPU).

The per-rank compute is the oracle (there is no GPU here); what is tested is
the host logic of fame_gb300.sharded: chunk assignment, the summed strand vote
of chunk 0 and the summed tallies, which must reproduce the single-process
reference results exactly."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


class _OracleMatcher:
    def __init__(self, oi):
        self.oi = oi
        self.meth = np.zeros(4 * oi.n_cpg, np.uint16)

    def match(self, seq, offs, flags):
        m, iv, c = self.oi.match_chunk(seq, offs, bool(flags & 1), bool(flags & 2), bool(flags & 4), self.meth)
        return m, iv, c

    def tallies(self, reset=True):
        out = self.meth.reshape(-1, 4).copy()
        if reset:
            self.meth[:] = 0
        return out


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, golden_path, both, outdir):
    import torch.distributed as dist
    from conftest import split_genome
    from fame_gb300.sharded import sharded_query
    from oracle.oracle import OracleIndex
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = dict(np.load(golden_path, allow_pickle=True))
    oi = OracleIndex.build(split_genome(g), readlen=100)
    (ids, mats, inv), meth, cnt = sharded_query(g["read_seq"].tobytes(), g["read_offs"], _OracleMatcher(oi), rank,
                                                world, dist=dist, chunk=1000 if not both else 777, both_strands=both)
    np.savez(os.path.join(outdir, "rank%d.npz" % rank), ids=ids, mats=mats, inv=inv, meth=meth, cnt=cnt)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("both,name", [(False, "chunk1000"), (True, "both")])
def test_two_rank_sharding_reproduces_reference(golden, tmp_path, both, name):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), os.path.join(here, "golden", "se_small.npz"), both, str(tmp_path)),
             nprocs=world, join=True)
    n = len(golden["read_offs"]) - 1
    mats = np.zeros(n, np.uint64)
    inv = np.full(n, 255, np.uint8)
    metas, cnts = [], []
    for r in range(world):
        d = np.load(tmp_path / ("rank%d.npz" % r))
        mats[d["ids"]] = d["mats"]
        inv[d["ids"]] = d["inv"]
        metas.append(d["meth"])
        cnts.append(d["cnt"])
    assert (inv != 255).all()
    assert np.array_equal(metas[0], metas[1]) and np.array_equal(cnts[0], cnts[1])
    assert np.array_equal(mats, golden[name + "_mat"])
    assert np.array_equal(inv, golden[name + "_invalid"])
    assert np.array_equal(metas[0], golden[name + "_meth"])
    assert np.array_equal(cnts[0], golden[name + "_counters"])
