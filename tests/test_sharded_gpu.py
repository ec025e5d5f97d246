"""The per-rank kernel of row sharding (nbgb_force_rows) on one GB300: any
split of the target rows assembles the full force (within the force gates;
different row counts plan different j-splits, so rounding may differ), and a
one-rank ShardedSystem steps exactly like the resident System."""
import os
import socket

import numpy as np
import pytest

from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

TOL_VS_REFERENCE = 1e-5
TOL_VS_FP64 = 5e-6


@pytest.mark.parametrize("n,cuts", [(16384, [0, 8192, 16384]), (10007, [0, 1, 3335, 6670, 10007]),
                                    (4096, [0, 4096])])
def test_row_slices_assemble_the_full_force(cuda, n, cuts):
    import torch
    pm_np, _ = nb.ic_uniform_ball(n, 70 + n, 1.0, 0.5, 1.5)
    pm = torch.from_numpy(pm_np).cuda()
    parts = [nb.force_rows(pm, 1e-4, a, b) for a, b in zip(cuts[:-1], cuts[1:])]
    torch.cuda.synchronize()
    assert nb.last_status() == 0
    out = torch.cat(parts).cpu().numpy()
    assert out.shape == (n, 4)
    ref = O.ieee().forces_aos(pm_np, 1e-4)
    assert O.per_body_rel_error(out, ref)[0] <= TOL_VS_REFERENCE
    f64 = np.zeros((n, 4))
    f64[:, :3] = O.ieee().forces_f64(pm_np, float(np.float32(1e-4)))
    assert O.per_body_rel_error(out, f64)[0] <= TOL_VS_FP64


def test_row_argument_errors(cuda):
    import torch
    lib = nb.load()
    pm = torch.zeros((64, 4), device="cuda")
    f = torch.zeros((64, 4), device="cuda")
    assert lib.nbgb_force_rows(f.data_ptr(), pm.data_ptr(), 1e-4, 64, 10, 70, None, 0,
                               None) == -1
    assert lib.nbgb_force_rows(f.data_ptr(), pm.data_ptr(), 1e-4, 64, 10, 5, None, 0, None) == -1
    assert lib.nbgb_force_rows(f.data_ptr(), pm.data_ptr(), 1e-4, 64, 7, 7, None, 0, None) == 0
    assert lib.nbgb_force_rows(f.data_ptr(), pm.data_ptr(), 1e-4, 64, 0, 64, None, 0, None) == -2


def test_one_rank_sharded_system_equals_resident_system(cuda):
    import torch
    import torch.distributed as dist
    from nbody_gb300.sharded import ShardedSystem
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=0, world_size=1)
    try:
        n = 5000
        pm0, vm0 = nb.ic_reference(n, 7)
        sh = ShardedSystem(n, 0.01, 0.016, 0.95, fused_drift=True)
        sh.set_state(pm0, vm0)
        sh.step(4)
        p_sh, v_sh = sh.get_state()
        sysm = nb.System(n, nb.INTEGRATOR_REFERENCE_FUSED, 0.01, 0.016, 0.95)
        sysm.set_state(pm0, vm0)
        sysm.step(4)
        p, v = sysm.get_state()
        sysm.close()
        torch.cuda.synchronize()
        assert np.array_equal(p_sh, p) and np.array_equal(v_sh, v)
    finally:
        dist.destroy_process_group()
