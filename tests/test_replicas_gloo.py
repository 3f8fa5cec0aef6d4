"""The multi-GPU path of bench.py is replicas only (the workload does not
shard): each rank runs its own copy, the job time is the max over ranks and
the work the sum.  Checked here with two gloo ranks on the CPU, each running
the oracle's force loop on its own plate."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    import time

    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import oracle as orc

    orc.set_threads(1)
    p = orc.derive_params(2, 1, 2, 1e-8, 10, 5e-5, 0.0, 5e-5, 0.002 * (rank + 1), 0.002, 0.0, 72e9, 1 / 3, 2440,
                          7e-4)
    x, y = orc.plate_coords(p)
    m = orc.Model(p, x, y)
    m.find_neighbor()
    m.surface_correct()
    t0 = time.perf_counter()
    for _ in range(3 + rank):  # unequal work per rank
        m.explicit_step()
    elapsed = time.perf_counter() - t0
    work = int(m.NN.sum()) * (3 + rank)
    secs, total = bench.aggregate_replicas(elapsed, work, dist, "cpu")
    q.put((rank, elapsed, work, secs, total))
    dist.destroy_process_group()


def test_two_gloo_replicas_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    (r0, e0, w0, s0, t0), (r1, e1, w1, s1, t1) = res
    assert s0 == s1 == pytest.approx(max(e0, e1))
    assert t0 == t1 == w0 + w1
    assert w1 > w0
