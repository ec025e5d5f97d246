"""Row sharding across ranks (nbody_gb300.sharded), the counterpart of the
reference's multi-GPU algorithm (src/nbody_multiGPU.cu:47-140), on CPU with
gloo: each rank evaluates its rows with the oracle's CPU_AOS restatement in
place of the GPU kernel and integrates them with the oracle's integrator;
the assembled trajectory and forces must equal the single-process oracle
bit for bit (the partition, the exchange order and the row bookkeeping are
what is under test).  World sizes 2 and 3, ragged N and an empty last rank."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import ROOT

EPS2, DT, DAMPING = 1e-4, 0.01, 0.95


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _bodies(n):
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    pm, vm = O.ieee().random_unit_bodies(n, 3)
    return pm, vm


def _worker(rank, ws, port, n, steps, fused, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import sys
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from nbody_gb300.sharded import ShardedSystem, row_range, sharded_force
    from oracle import oracle as O

    def force_rows(pm, eps2, r0, r1, out):
        out[:] = torch.from_numpy(O.ieee().forces_aos_idx(pm.numpy(), eps2, np.arange(r0, r1)))

    def integrate(pm_rows, vel_rows, f_rows, dt, damping, fused_drift):
        fn = O.ieee().integrate_contracted if fused_drift else O.ieee().integrate
        fn(pm_rows.numpy(), vel_rows.numpy(), f_rows.numpy(), dt, damping)

    pm0, vm0 = _bodies(n)
    f = sharded_force(torch.from_numpy(pm0), EPS2, force_rows_fn=force_rows).numpy().copy()
    s = ShardedSystem(n, EPS2, DT, DAMPING, device=torch.device("cpu"), fused_drift=fused,
                      force_rows_fn=force_rows, integrate_fn=integrate)
    s.set_state(pm0, vm0)
    s.step(steps)
    p, v = s.get_state()
    rows = row_range(n, ws, rank)
    dist.destroy_process_group()
    q.put((rank, rows, f, p, v))


@pytest.mark.timeout(180)
@pytest.mark.parametrize("ws,n,fused", [(2, 1001, False), (2, 1024, True), (3, 5, False),
                                        (3, 4, True)])
def test_row_sharded_steps_equal_single_process(ws, n, fused):
    steps = 3
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, n, steps, fused, q))
             for r in range(ws)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=150) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0

    from oracle import oracle as O
    pm0, vm0 = _bodies(n)
    f_ref = O.ieee().forces_aos(pm0, EPS2)
    p, v = pm0.copy(), vm0.copy()
    for _ in range(steps):
        f = O.ieee().forces_aos(p, EPS2)
        (O.ieee().integrate_contracted if fused else O.ieee().integrate)(p, v, f, DT, DAMPING)
    covered = []
    for rank, (r0, r1, r), fs, ps, vs in out:
        covered.extend(range(r0, r1))
        assert np.array_equal(fs[:, :3], f_ref[:, :3])
        assert np.array_equal(ps, p) and np.array_equal(vs[:, :3], v[:, :3])
        assert np.array_equal(vs[:, 3], v[:, 3])
    assert covered == list(range(n))  # every row owned by exactly one rank, in order
