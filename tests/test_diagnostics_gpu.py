"""Potential mode of the force kernel, FP64 conserved-quantity reductions and
a short precision-study run, against the oracle's FP64 sums."""
import numpy as np
import pytest

from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

POT_CONFIG = 23


def test_potential_mode_matches_fp64(cuda):
    import torch
    n = 5000
    _, _, pm, _ = nb.ic_plummer(n, 12)
    eps2 = float(np.float32(1e-4))
    for nsplit in (1, 3):
        out = nb.force(torch.from_numpy(pm).cuda(), 1e-4, config=POT_CONFIG,
                       nsplit=nsplit).cpu().numpy()
        phi = O.ieee().potential_f64(pm, eps2)
        f = np.zeros((n, 4))
        f[:, :3] = O.ieee().forces_f64(pm, eps2)
        assert O.per_body_rel_error(out, f)[0] <= 5e-6
        rel = np.abs(out[:, 3] - phi) / np.abs(phi)
        assert rel.max() <= 2e-6


def _oracle_energy(pm4, vel3, m):
    phi = O.ieee().potential_f64(pm4, float(np.float32(1e-4)))
    return 0.5 * (m * (vel3 ** 2).sum(1)).sum(), 0.5 * (m * phi).sum()


def test_system_diagnostics_kdk(cuda):
    n = 4096
    p, v, pm, _ = nb.ic_plummer(n, 13)
    m = pm[:, 3].astype(np.float64)
    s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, 0.002, 1.0)
    s.set_state64(p, v, pm[:, 3].copy())
    d = s.diagnostics()
    ke, pe = _oracle_energy(pm, v, m)
    assert abs(d["kinetic"] - ke) <= 1e-12 * abs(ke)
    assert abs(d["potential"] - pe) <= 2e-6 * abs(pe)
    mom = (m[:, None] * v).sum(0)
    assert np.allclose(d["momentum"], mom, rtol=0, atol=1e-14)
    ang = (m[:, None] * np.cross(p, v)).sum(0)
    assert np.allclose(d["angular_momentum"], ang, rtol=0, atol=1e-13)
    # deterministic
    assert s.diagnostics()["potential"] == d["potential"]
    s.close()


def test_system_diagnostics_reference_mode(cuda):
    pm, vm = nb.ic_reference(2048, 7)
    s = nb.System(2048, nb.INTEGRATOR_REFERENCE, 0.01, 0.016, 0.95)
    s.set_state(pm, vm)
    d = s.diagnostics()
    m = pm[:, 3].astype(np.float64)
    v = vm[:, :3].astype(np.float64)
    phi = O.ieee().potential_f64(pm, float(np.float32(0.01)))
    assert abs(d["kinetic"] - 0.5 * (m * (v ** 2).sum(1)).sum()) <= 1e-12 * d["kinetic"]
    assert abs(d["potential"] - 0.5 * (m * phi).sum()) <= 2e-6 * abs(d["potential"])
    s.close()


def test_short_precision_study(cuda):
    from nbody_gb300.studies import precision_study
    r = precision_study(n=8192, steps=200, dt=0.002, eps2=1e-4, seed=3, n_sample=512, every=50)
    assert r["force_error_start"]["max"] <= 5e-6 and r["force_error_end"]["max"] <= 5e-6
    assert r["force_error_start"]["rms"] <= 1e-6
    assert r["energy_drift_max"] < 1e-4
    assert np.abs(r["momentum_end"]).max() < 1e-6
