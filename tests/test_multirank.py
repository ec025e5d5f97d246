"""The N>1 path of bench.py (independent replicas, one per GPU) on CPU with
gloo and world_size 2: barrier, slowest-rank time, summed work, and the
reference arm's rank > 0 exiting without work."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(ws),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    w, r, local = bench._dist()
    assert (w, r, local) == (ws, rank, rank)
    bench._barrier(w)
    # rank k took (k + 1) seconds for (k + 1) * 1e9 interactions
    value, t_max, total = bench.aggregate(w, float(rank + 1), float(rank + 1) * 1e9)
    # reference arm: only rank 0 prints / works
    class A:
        steps, warmup = 1, 0
    printed = None
    if rank != 0:
        printed = bench.run_reference_arm(A, w, rank)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((rank, value, t_max, total, printed))


@pytest.mark.timeout(120)
def test_replica_aggregation_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, value, t_max, total, printed in out:
        assert t_max == 2.0 and total == 3e9 and abs(value - 1.5) < 1e-12
        assert printed is None
