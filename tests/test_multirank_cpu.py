"""The multi-rank bench path on CPU: two gloo ranks split the replicated system list with
the product's partitioner (csem_partition_systems; disjoint units, equal expected work,
no exchange of solver data) and agree on the max-over-ranks timing."""
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    from demo_matrixfree_csem_gb300 import synthetic
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = synthetic.random_small(5, freqs=(0.5, 1.0))
    cfg.acq.src = np.repeat(cfg.acq.src, 3, axis=0)
    cfg.acq.src[:, 0] += 100.0 * np.arange(3)
    systems = [(f, s) for f in (0.5, 1.0) for s in range(3)]
    mine = bench.rank_systems(systems, world, rank, 1000)
    waves = [bench.wave_systems(cfg, mine, 4, k) for k in range(2)]
    wall = bench.max_over_ranks([1.0 + rank, 5.0 - rank], "cpu")
    out[rank] = (waves, wall, mine)
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_gloo_ranks_partition_and_reduce():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        out = man.dict()
        port = _free_port()
        ps = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    (w0, t0, m0), (w1, t1, m1) = res[0], res[1]
    assert t0 == t1 == [2.0, 5.0]                        # max over ranks, seen by every rank
    assert not set(m0) & set(m1)                         # disjoint units
    assert len(set(m0) | set(m1)) == 12                  # together: both copies of the 6 systems
    assert sorted(f for f, _, _ in m0) == sorted(f for f, _, _ in m1)  # the same work on each rank
    for (f0, s0), (f1, s1) in zip(w0, w1):
        assert not np.any(np.all(s0[:, None] == s1[None], axis=2))  # disjoint source positions
    assert [len(f) for f, _ in w0] == [4, 2]             # 6 systems in waves of 4
