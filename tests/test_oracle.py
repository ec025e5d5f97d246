"""Pins the CPU oracle to the reference's own outputs (tests/golden/, made by
the reference's compiled CPU_AOS / CPU_SOA / randomUnitBodies objects)."""
import numpy as np
import pytest

from conftest import GOLDEN_FORCE_CASES, golden
from oracle import oracle as O

# Per-body norm-wise tolerance of an FP32 all-pairs force against the
# reference's CPU_AOS (the per-body accuracy gate of the force path).
FORCE_TOL = 1e-5


@pytest.mark.parametrize("case", GOLDEN_FORCE_CASES)
def test_restatement_matches_reference_forces(case):
    g = golden(case)
    pm, eps2 = g["posMass"], float(g["eps2"])
    for impl in (O.ieee(), O.fast()):
        f = impl.forces_aos(pm, eps2)
        mx, rms = O.per_body_rel_error(f, g["force_aos"])
        assert mx <= FORCE_TOL, (case, mx, rms)
    f = O.fast().forces_soa(pm, eps2)
    assert O.per_body_rel_error(f, g["force_aos"])[0] <= FORCE_TOL


@pytest.mark.parametrize("case", GOLDEN_FORCE_CASES)
def test_fp64_oracle_matches_reference(case):
    g = golden(case)
    f = O.ieee().forces_f64(g["posMass"], float(g["eps2"]))
    ref = g["force_aos"].astype(np.float64)[:, :3]
    num = np.linalg.norm(ref - f, axis=1)
    den = np.linalg.norm(f, axis=1)
    assert (num / den).max() <= FORCE_TOL
    # the stored FP64 forces are this oracle's (regression guard)
    np.testing.assert_allclose(f, g["force_f64"][:, :3], rtol=0, atol=0)


def test_reference_aos_and_soa_agree():
    g = golden("ball2048")
    assert np.array_equal(g["force_aos"][:, :3], g["force_soa"][:, :3])


def test_reference_initial_conditions_exact():
    g = golden("refic1024_seed7")
    pos, vel = O.ieee().random_unit_bodies(1024, 7, 0.9, 8.0)
    assert np.array_equal(pos, g["posMass"])
    assert np.array_equal(vel, g["velInvMass"])


def test_integrator_restatement_reproduces_trajectory_step():
    t = golden("traj1024")
    p, v = t["posMass0"].copy(), t["velInvMass0"].copy()
    f = t["force_step1"].copy()
    O.ieee().integrate(p, v, f, float(t["dt"]), float(t["damping"]))
    assert np.array_equal(p, t["posMass1"])
    assert np.array_equal(v, t["velInvMass1"])


def test_crosscheck_metric_semantics():
    # relError(a, b) = |a-b|/b with signed b: negative-golden components never
    # raise the maximum (src/nbody.cu:120-125)
    g = np.zeros((2, 4), np.float32)
    f = np.zeros((2, 4), np.float32)
    g[0, :3] = [1.0, -1.0, 2.0]
    f[0, :3] = [1.1, -2.0, 2.0]
    g[1, :3] = [4.0, 0.0, 0.0]
    f[1, :3] = [4.0, 0.0, 0.0]
    f[1, 3] = 99.0  # w is ignored
    e = O.ieee().max_rel_error(f, g)
    assert abs(e - 0.1) < 1e-6


def test_plain_16k_fixture_restatement():
    """The exact plain single-system case (N = 16,384 unit ball, m = 1/N,
    eps2 = 1e-4): the IEEE restatement of CPU_AOS is within the per-body gate
    of the reference's own CPU_AOS forces, and the reference integrator as the
    reference binary computes it (position update fused) reproduces the
    reference driver's compiled integrateGravitation_SOA bit for bit."""
    g = golden("c1_ball16384")
    f = O.ieee().forces_aos(g["posMass0"], float(g["eps2"]))
    assert O.per_body_rel_error(f, g["force_aos0"])[0] <= FORCE_TOL
    p, v = g["posMass0"].copy(), g["velInvMass0"].copy()
    O.ieee().integrate_contracted(p, v, g["force_aos0"].copy(), float(g["dt"]),
                                  float(g["damping"]))
    assert np.array_equal(p, g["posMass1"]) and np.array_equal(v, g["velInvMass1"])
    # the separately rounded form differs from the compiled reference only in
    # the position update
    p2, v2 = g["posMass0"].copy(), g["velInvMass0"].copy()
    O.ieee().integrate(p2, v2, g["force_aos0"].copy(), float(g["dt"]), float(g["damping"]))
    assert np.array_equal(v2, g["velInvMass1"])


def test_forces_for_listed_targets_match_full_sum():
    g = golden("plummer4096")
    idx = np.array([0, 1, 777, 4095, 2048, 777])
    for impl in (O.ieee(), O.fast()):
        full = impl.forces_aos(g["posMass"], float(g["eps2"]))
        part = impl.forces_aos_idx(g["posMass"], float(g["eps2"]), idx)
        assert np.array_equal(part[:, :3], full[idx, :3])


@pytest.mark.parametrize("n,seed", [(1, 3), (1000, 20260), (4097, 2 ** 61 + 5), (65536, 9)])
def test_plummer_restatement_is_byte_identical(n, seed):
    """The CPU baseline builds its Plummer inputs with the oracle's
    restatement of the library's generator, without loading the library:
    both must give the same bytes."""
    import nbody_gb300 as nb
    p, v, pm = O.ieee().ic_plummer(n, seed)
    p2, v2, pm2, _ = nb.ic_plummer(n, seed)
    assert np.array_equal(p, p2) and np.array_equal(v, v2) and np.array_equal(pm, pm2)


def test_million_body_fixture():
    """The plain large system's input regenerates from its seed (the oracle's
    restatement of the library's Plummer generator) to the fixture's bytes,
    and the reference's compiled CPU_AOS forces stored for its sample are
    within the gate of the FP64 sum and of the restatement built with the
    reference's flags."""
    import hashlib
    g = golden("c2_plummer1m_sample")
    _, _, pm = O.ieee().ic_plummer(int(g["n"]), int(g["seed"]))
    assert hashlib.sha256(pm.tobytes()).hexdigest() == g["posMass_sha256"].item().decode()
    assert np.array_equal(pm[g["idx"]], g["posMass_idx"])
    ref = g["force_aos"][:, :3].astype(np.float64)
    d = np.linalg.norm(ref - g["force_f64"], axis=1) / np.linalg.norm(g["force_f64"], axis=1)
    assert d.max() <= FORCE_TOL
    f = O.fast().forces_aos_idx(pm, float(g["eps2"]), g["idx"])
    assert O.per_body_rel_error(f, g["force_aos"])[0] <= FORCE_TOL
