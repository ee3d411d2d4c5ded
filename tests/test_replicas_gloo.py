"""Multi-rank path of bench.py on CPU: two gloo ranks, independent replicas.

Each rank simulates its own replica with the oracle (seeded by rank), the
aggregation takes the max time and the summed events, and the whole-job
realtime factor counts every replica's biological time.
"""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "cerebellar-scaffold-model-simulation-on-gpu_gb300"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle_py
    import scaffold_gb300 as sg

    net = sg.scaffold(1, 0.1, 1 + rank)
    o = oracle_py.Oracle(oracle_py.describe(net), seed=1 + rank)
    counts, _ = o.run(200)
    ms = 10.0 * (rank + 1)  # rank 1 is the slowest replica
    ms_max, ev = bench.aggregate(dist, "cpu", ms, float(o.events()))
    q.put((rank, ms_max, ev, int(o.events()), int(counts.sum())))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    (_, m0, e0, own0, c0), (_, m1, e1, own1, c1) = out
    assert m0 == m1 == 20.0                       # max over ranks
    assert e0 == e1 == float(own0 + own1)          # sum over ranks
    assert c0 > 0 and c1 > 0 and (own0, c0) != (own1, c1)  # different replicas
    import bench
    assert bench.realtime_factor(2, 3, 0.1, 20.0) == pytest.approx(30.0)
