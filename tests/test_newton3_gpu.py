"""The Newton's-third-law force variant against the reference's fixtures, the
oracle, FP64 and the one-sided kernel."""
import numpy as np
import pytest

from conftest import GOLDEN_FORCE_CASES, golden
from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

TOL_VS_REFERENCE = 1e-5
TOL_VS_FP64 = 5e-6


def _n3(pm, eps2):
    import torch
    out = nb.force_newton3(torch.from_numpy(np.ascontiguousarray(pm, np.float32)).cuda(), eps2)
    torch.cuda.synchronize()
    assert nb.last_status() == 0
    return out.cpu().numpy()


def _f64(pm, eps2, idx=None):
    f = O.ieee().forces_f64(pm, float(np.float32(eps2)), idx)
    o = np.zeros((f.shape[0], 4))
    o[:, :3] = f
    return o


@pytest.mark.parametrize("case", GOLDEN_FORCE_CASES)
def test_matches_reference_fixtures(cuda, case):
    g = golden(case)
    out = _n3(g["posMass"], float(g["eps2"]))
    assert np.all(out[:, 3] == 0)
    assert O.per_body_rel_error(out, g["force_aos"])[0] <= TOL_VS_REFERENCE
    assert O.per_body_rel_error(out, g["force_f64"])[0] <= TOL_VS_FP64


@pytest.mark.parametrize("n", [1, 2, 127, 128, 129, 1023, 1024, 1025, 3000, 5000])
def test_ragged_sizes(cuda, n):
    pm, _ = nb.ic_uniform_ball(n, 500 + n, 1.0, 0.5, 1.5)
    out = _n3(pm, 1e-4)
    if n == 1:
        assert np.all(out[0, :3] == 0)
        return
    assert O.per_body_rel_error(out, _f64(pm, 1e-4))[0] <= TOL_VS_FP64


def test_large_plummer_against_fp64_and_momentum(cuda):
    n = 1 << 18
    _, _, pm, _ = nb.ic_plummer(n, 33)
    out = _n3(pm, 1e-4)
    idx = np.random.default_rng(3).choice(n, 512, replace=False)
    mx, rms = nb.force_error_stats(out, _f64(pm, 1e-4, idx)[:, :3], idx)
    assert mx <= TOL_VS_FP64 and rms <= 1e-6
    m = pm[:, 3:4].astype(np.float64)
    tot = (m * out[:, :3]).sum(0)
    scale = (m * np.abs(out[:, :3])).sum(0)
    assert np.all(np.abs(tot) <= 1e-6 * scale)  # pairs cancel up to FP32 rounding


def test_resident_system_with_newton3(cuda):
    n = 4096
    p, v, pm, _ = nb.ic_plummer(n, 8)
    m = pm[:, 3].copy()
    out = []
    for algo in ("onesided", "newton3"):
        s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, 0.002, 1.0)
        s.set_force_algorithm(algo)
        s.set_state64(p, v, m)
        s.step(20)
        out.append(s.get_state64())
        s.close()
    (p1, v1), (p2, v2) = out
    # the one-sided plan takes every fourth source pair in the log domain
    # (per-term error a few times the rsqrt form's): after 20 steps the
    # velocities agree to small multiples of the FP32 force error times dt
    assert np.abs(p1 - p2).max() <= 1e-9 * np.abs(p1).max()
    assert np.abs(v1 - v2).max() <= 5e-8 * np.abs(v1).max()


def test_drop_in_row(cuda):
    import torch
    g = golden("ball2048")
    pm = torch.from_numpy(g["posMass"]).cuda()
    f = torch.full_like(pm, 3.0)
    ms = nb.ComputeGravitation_GPU_GB300_Newton3(f, pm, float(g["eps2"]), pm.shape[0])
    assert ms > 0.0
    out = f.cpu().numpy()
    assert O.per_body_rel_error(out, g["force_aos"])[0] <= TOL_VS_REFERENCE
    assert nb.ComputeGravitation_GPU_GB300_Newton3(f, pm, 1e-4, 0) == 0.0
