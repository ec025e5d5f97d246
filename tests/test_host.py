"""Host-side library code (no GPU): the FP64 self-check against the oracle's
FP64 sum, and the initial-condition generators' statistics."""
import numpy as np

from oracle import oracle as O

import nbody_gb300 as nb


def test_force_f64_host_matches_oracle():
    _, _, pm, _ = nb.ic_plummer(6000, 9)
    idx = np.arange(0, 6000, 37)
    eps2 = float(np.float32(1e-4))
    f, phi = nb.force_f64_host(pm, 1e-4, idx)
    f2 = O.ieee().forces_f64(pm, eps2, idx)
    p2 = O.ieee().potential_f64(pm, eps2, idx)
    assert np.allclose(f, f2, rtol=1e-13, atol=0)
    assert np.allclose(phi, p2, rtol=1e-13, atol=0)


def test_force_f64_host_rejects_bad_index():
    pm = np.zeros((10, 4), np.float32)
    import pytest
    with pytest.raises(nb.NbgbError):
        nb.force_f64_host(pm, 1e-4, np.array([10]))


def test_plummer_statistics():
    p, v, pm, vm = nb.ic_plummer(50000, 1)
    r = np.linalg.norm(p, axis=1)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.305
    assert abs(np.median(r) - 1.305) < 0.03
    ke = 0.5 * (v ** 2).sum() / 50000
    assert abs(ke - 3 * np.pi / 64) < 0.01  # virial: K = 3 pi / 64 (G = M = a = 1)
    assert np.abs(p.mean(0)).max() < 1e-12 and np.abs(v.mean(0)).max() < 1e-12
    assert np.all(pm[:, 3] == np.float32(1 / 50000))
    assert np.array_equal(pm[:, :3], p.astype(np.float32))


def test_uniform_ball_statistics():
    pm, vm = nb.ic_uniform_ball(40000, 2, 1.0, 0.5, 1.5)
    r = np.linalg.norm(pm[:, :3].astype(np.float64), axis=1)
    assert r.max() <= 1.0 + 1e-6
    assert abs(np.median(r) - 0.5 ** (1 / 3)) < 0.01  # uniform ball: P(r < R) = R^3
    m = pm[:, 3] * 40000
    assert 0.5 - 1e-4 <= m.min() and m.max() <= 1.5 + 1e-4
    assert np.all(vm[:, :3] == 0) and np.allclose(vm[:, 3], 1 / pm[:, 3])


def test_generators_are_deterministic():
    a = nb.ic_plummer(1000, 5)
    b = nb.ic_plummer(1000, 5)
    c = nb.ic_plummer(1000, 6)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[0], c[0])


def test_reference_line_format():
    # src/nbody.cu:1033-1052
    line = nb.reference_line("GPU_GB300", 16384, 0.1, 1e-6, 13)
    assert line == ("    GPU_GB300:     0.10 ms = 2684.355x10^9 interactions/s "
                    "( 53687.09 GFLOPS) (Rel. error: 1.000000E-06)")
