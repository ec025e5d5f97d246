"""Device-resident step loop: the reference's crosscheck applied every step
(forces on identical positions, src/nbody.cu:313-325, 406-418), the fused
integrate bit-exact, and whole trajectories within the spread that the
reference's own CPU variants show."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

TOL_FORCE = 1e-5
# against FP64 on the same FP32 positions (see test_force_gpu.py)
TOL_VS_FP64 = 5e-6


def _rel_pos(a, b):
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)


def test_plain_case_ten_steps_crosschecked_every_step(cuda):
    """N = 16,384 unit ball, m = 1/N, v = 0, eps2 = 1e-4, dt = 0.01, 10 steps.
    Every step the GPU forces are compared on the same positions with an FP64
    all-pairs sum and with the IEEE binary32 restatement of CPU_AOS: the GPU
    must be within 5e-6 of FP64 or at least as close as the restatement
    (whose own error grows as the reference integrator scatters the bodies),
    and within 1e-5 of the restatement itself."""
    n = 16384
    pm0, vm0 = nb.ic_uniform_ball(n, 16384)
    sysm = nb.System(n, nb.INTEGRATOR_REFERENCE, 1e-4, 0.01, 0.95)
    sysm.set_state(pm0, vm0)
    eps2 = float(np.float32(1e-4))
    for step in range(10):
        p_before, v_before = sysm.get_state()
        sysm.step(1)
        f_gpu = sysm.get_force()
        f_ieee = O.ieee().forces_aos(p_before, 1e-4)
        f64 = np.zeros((n, 4))
        f64[:, :3] = O.ieee().forces_f64(p_before, eps2)
        mx, rms = O.per_body_rel_error(f_gpu, f64)
        mx_i, rms_i = O.per_body_rel_error(f_ieee, f64)
        assert mx <= max(TOL_VS_FP64, mx_i) and rms <= rms_i, (step, mx, mx_i, rms, rms_i)
        assert O.per_body_rel_error(f_gpu, f_ieee)[0] <= max(TOL_FORCE, 2 * mx_i), step
        # the fused integrate on the GPU forces: bit-exact
        O.ieee().integrate(p_before, v_before, f_gpu, 0.01, 0.95)
        p_after, v_after = sysm.get_state()
        assert np.array_equal(p_after, p_before) and np.array_equal(v_after, v_before)
    sysm.close()


def test_plain_case_trajectory_within_reference_spread(cuda):
    """Free-running 10-step trajectory against the oracle-driven one (IEEE
    binary32 restatement; the restatement built with the reference's aarch64
    flags uses -mlow-precision-recip-sqrt and is itself 6e-5 off).  The
    reference's integrator multiplies the acceleration by 1/m = N, so
    rounding differences grow quickly; the reference's own CPU variants
    (CPU_AOS vs the IEEE restatement) differ at step 10 by median 2.4e-5,
    p99 2.4e-3 per body.  Bounds: step 1 max 1e-4; step 10 median 1e-4,
    p99 1e-2."""
    n = 16384
    pm0, vm0 = nb.ic_uniform_ball(n, 16384)
    sysm = nb.System(n, nb.INTEGRATOR_REFERENCE, 1e-4, 0.01, 0.95)
    sysm.set_state(pm0, vm0)
    p, v = pm0.copy(), vm0.copy()
    for step in range(1, 11):
        sysm.step(1)
        f = O.ieee().forces_aos(p, 1e-4)
        O.ieee().integrate(p, v, f, 0.01, 0.95)
        g, _ = sysm.get_state()
        rel = _rel_pos(g, p)
        if step == 1:
            assert rel.max() <= 1e-4
    assert np.median(rel) <= 1e-4 and np.quantile(rel, 0.99) <= 1e-2
    sysm.close()


def test_golden_trajectory(cuda):
    t = golden("traj1024")
    sysm = nb.System(1024, nb.INTEGRATOR_REFERENCE, float(t["eps2"]), float(t["dt"]),
                     float(t["damping"]))
    sysm.set_state(t["posMass0"], t["velInvMass0"])
    sysm.step(1)
    p1, _ = sysm.get_state()
    assert _rel_pos(p1, t["posMass1"]).max() <= 1e-4
    sysm.step(4)
    p5, _ = sysm.get_state()
    sysm.step(5)
    p10, _ = sysm.get_state()
    for p, ref in ((p5, t["posMass5"]), (p10, t["posMass10"])):
        rel = _rel_pos(p, ref)
        assert np.median(rel) <= 1e-4 and np.quantile(rel, 0.99) <= 1e-2
    sysm.close()


def test_graph_and_eager_steps_identical(cuda):
    pm0, vm0 = nb.ic_reference(4096, 7)
    out = []
    for graph in (True, False):
        s = nb.System(4096, nb.INTEGRATOR_REFERENCE, 0.01, 0.016, 0.95)
        s.use_graph(graph)
        s.set_state(pm0, vm0)
        s.step(19)  # two 8-step graphs and three direct steps
        out.append(s.get_state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_kdk64_graph_and_eager_steps_identical(cuda):
    n = 3000
    p, v, pm, _ = nb.ic_plummer(n, 5)
    out = []
    for graph in (True, False):
        s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, 0.002, 1.0)
        s.use_graph(graph)
        s.set_state64(p, v, pm[:, 3].copy())
        s.step(20)  # an opening step, two 8-step graphs, three direct steps
        s.step(9)   # a merged opening kick, one graph
        out.append(s.get_state64())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_kdk64_conserves_energy_small(cuda):
    """FP64 leapfrog on a 2,048-body Plummer sphere: energy drift over 200
    steps at dt = 0.002 stays small (FP64 energy from the oracle)."""
    n = 2048
    p, v, pm, _ = nb.ic_plummer(n, 3)
    m = pm[:, 3].copy()
    s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, 0.002, 1.0)
    s.set_state64(p, v, m)

    def energy(pos, vel):
        pm4 = np.zeros((n, 4), np.float32)
        pm4[:, :3] = pos
        pm4[:, 3] = m
        phi = O.ieee().potential_f64(pm4, float(np.float32(1e-4)))
        return 0.5 * (m * (vel ** 2).sum(1)).sum() + 0.5 * (m * phi).sum()

    e0 = energy(p, v)
    s.step(200)
    p1, v1 = s.get_state64()
    e1 = energy(p1, v1)
    assert abs(e1 - e0) / abs(e0) < 1e-4
    # momentum stays ~0
    assert np.abs((m[:, None] * v1).sum(0)).max() < 1e-6
    s.close()


def test_negative_masses_replan_the_system(cuda):
    """A system whose plan takes some source pairs in the log domain moves to
    an rsqrt-only plan when masses < 0 are set, and its forces then follow the
    reference's formula for any sign."""
    n = 3000
    pm0, vm0 = nb.ic_uniform_ball(n, 99, 1.0, 0.5, 1.5)
    pm0 = pm0.copy()
    pm0[0, 3] = -pm0[0, 3]
    sysm = nb.System(n, nb.INTEGRATOR_REFERENCE, 1e-4, 0.01, 0.95)
    sysm.set_state(pm0, vm0)
    cfg, _ = sysm.plan()
    assert not nb.force_config_names()[cfg].endswith("log4")
    p_before, _ = sysm.get_state()
    sysm.step(1)
    sysm.synchronize()
    f = sysm.get_force()
    ref = O.ieee().forces_aos(p_before, 1e-4)
    assert O.per_body_rel_error(f, ref)[0] <= TOL_FORCE
    # the replanned system keeps stepping through both j-stream buffers
    for _ in range(3):
        p_before, v_before = sysm.get_state()
        sysm.step(1)
        f = sysm.get_force()
        assert O.per_body_rel_error(f, O.ieee().forces_aos(p_before, 1e-4))[0] <= TOL_FORCE
        O.ieee().integrate(p_before, v_before, f, 0.01, 0.95)
        p_after, v_after = sysm.get_state()
        assert np.array_equal(p_after, p_before) and np.array_equal(v_after, v_before)
    sysm.close()


def _host_steps(p, v, m, fused, fn):
    """m reference steps on host copies: forces by fn(p) on the GPU, then the
    oracle's integrator (separately rounded or contracted drift)."""
    import torch
    f = None
    for _ in range(m):
        f = fn(torch.from_numpy(p).cuda()).cpu().numpy()
        (O.ieee().integrate_contracted if fused else O.ieee().integrate)(p, v, f, 0.016, 0.95)
    return f


@pytest.mark.parametrize("n,integrator", [(1000, nb.INTEGRATOR_REFERENCE),
                                          (10007, nb.INTEGRATOR_REFERENCE_FUSED),
                                          (65536, nb.INTEGRATOR_REFERENCE),
                                          (155677, nb.INTEGRATOR_REFERENCE_FUSED)])
def test_fused_epilogue_step_is_force_then_integrate(cuda, n, integrator):
    """A reference step on the one-sided kernel is one launch: the force
    kernel's epilogue integrates each body once its force is final and writes
    the next step's j-stream into the other of two buffers.  Every step must
    equal the standalone force kernel on that step's positions followed by the
    reference integrator, bit for bit: through graph launches (two graphs,
    one per starting buffer), eager and timed steps, a state reset between
    steps, and a detour through the Newton-3 algorithm (whose separate
    integrate writes the current buffer)."""
    fused = integrator == nb.INTEGRATOR_REFERENCE_FUSED
    pm0, vm0 = nb.ic_reference(n, 11)
    s = nb.System(n, integrator, 0.01, 0.016, 0.95)
    assert s.plan() == nb.force_plan(n)[:2]  # same plan as the standalone force()
    s.set_state(pm0, vm0)
    p, v = pm0.copy(), vm0.copy()

    def onesided(t):
        return nb.force(t, 0.01)

    def run(m, fn=onesided):
        f = _host_steps(p, v, m, fused, fn)
        s.step(m)
        ps, vs = s.get_state()
        assert np.array_equal(ps, p) and np.array_equal(vs, v), m
        assert np.array_equal(s.get_force()[:, :3], f[:, :3]), m

    for m in (1, 8, 1, 9, 16, 2):  # 8-step graphs from either buffer, direct steps
        run(m)
    s.use_graph(False)
    run(3)
    s.set_timing(True)
    run(1)
    assert s.last_force_ms() > 0.0
    with pytest.raises(nb.NbgbError):
        s.last_integrate_ms()  # the integrate ran inside the force launch
    s.set_timing(False)
    s.use_graph(True)
    pm1, vm1 = nb.ic_reference(n, 12)  # reset with the other buffer current
    s.set_state(pm1, vm1)
    p[:], v[:] = pm1, vm1
    run(1)
    run(8)
    s.set_force_algorithm("newton3")
    for _ in range(2):
        s.step(1)
        f = s.get_force()
        (O.ieee().integrate_contracted if fused else O.ieee().integrate)(p, v, f, 0.016, 0.95)
        ps, vs = s.get_state()
        assert np.array_equal(ps, p) and np.array_equal(vs, v)
    s.step(8)  # a Newton-3 graph
    p, v = s.get_state()
    s.set_force_algorithm("onesided")
    run(3)
    run(8)
    s.close()


@pytest.mark.parametrize("n", [1, 2, 3, 33, 257])
def test_tiny_systems_one_launch_steps(cuda, n):
    """Sizes far below one i-block or one j-tile (N = 1 has only its zero
    self term): ten one-launch reference steps, each equal to the oracle's
    CPU_AOS forces (within the force gate) and, on the GPU's own forces, the
    oracle's integrator bit for bit; graph and direct steps agree."""
    pm0, vm0 = nb.ic_reference(n, 3)
    out = []
    for graph in (True, False):
        s = nb.System(n, nb.INTEGRATOR_REFERENCE, 0.01, 0.016, 0.95)
        s.use_graph(graph)
        s.set_state(pm0, vm0)
        if graph:
            s.step(8)  # one graph, then per-step checks below
        for _ in range(2):
            p_before, v_before = s.get_state()
            s.step(1)
            f = s.get_force()
            ref = O.ieee().forces_aos(p_before, 0.01)
            if n == 1:
                assert np.all(f[:, :3] == 0)
            else:
                assert O.per_body_rel_error(f, ref)[0] <= TOL_FORCE
            O.ieee().integrate(p_before, v_before, f, 0.016, 0.95)
            p_after, v_after = s.get_state()
            assert np.array_equal(p_after, p_before) and np.array_equal(v_after, v_before)
        if not graph:
            s.step(8)  # the same ten steps in another order of launches
        out.append(s.get_state())
        s.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


def test_fused_epilogue_step_at_the_headline_size(cuda):
    """N = 2^20 (the plan takes whole i-blocks for the first rounds and splits
    the leftover i-blocks into many slices): two one-launch reference steps,
    each equal to the standalone force kernel on that step's positions and
    the reference integrator (contracted drift), bit for bit."""
    import torch
    n = 1 << 20
    _, _, pm0, vm0 = nb.ic_plummer(n, 2)  # velInvMass.w = 1/m
    s = nb.System(n, nb.INTEGRATOR_REFERENCE_FUSED, 1e-4, 0.005, 1.0)
    assert s.plan() == nb.force_plan(n)[:2]
    s.set_state(pm0, vm0)
    p, v = pm0.copy(), vm0.copy()
    for _ in range(2):
        f = nb.force(torch.from_numpy(p).cuda(), 1e-4).cpu().numpy()
        O.ieee().integrate_contracted(p, v, f, 0.005, 1.0)
        s.step(1)
        ps, vs = s.get_state()
        assert np.array_equal(ps, p) and np.array_equal(vs, v)
        assert np.array_equal(s.get_force()[:, :3], f[:, :3])
    s.close()


@pytest.mark.parametrize("config_name", ["w8_k4_jt512_s3_f32", "w8_k2_jt256_s4_f32x2",
                                         "w8_k2_jt256_s4_fma2", "w8_k4_jt256_s4_tpair",
                                         "w8_k2_jt1024_s3_log4", "w8_k2_jt1024_s2_pf_log4"])
@pytest.mark.parametrize("nsplit", [1, 3])
def test_fused_epilogue_in_every_kernel_mode(cuda, config_name, nsplit):
    """The integrate fused into the force epilogue under every kernel mode
    (scalar, f32x2, all-FMA, target pairs with the duplicated source layout,
    log-domain pairs, prefetching) and with and without a j-split, forced
    with System.set_plan: each step equals the standalone kernel of the same
    plan followed by the reference integrator, bit for bit."""
    n = 5003
    cfg = nb.force_config_names().index(config_name)
    pm0, vm0 = nb.ic_reference(n, 21)
    s = nb.System(n, nb.INTEGRATOR_REFERENCE, 0.01, 0.016, 0.95)
    s.set_plan(cfg, nsplit)
    assert s.plan() == nb.force_plan(n, cfg, nsplit)[:2]
    s.set_state(pm0, vm0)
    p, v = pm0.copy(), vm0.copy()

    def forced(t):
        return nb.force(t, 0.01, config=cfg, nsplit=nsplit)

    for m in (1, 2, 8):  # direct steps from either buffer, then one graph
        f = _host_steps(p, v, m, False, forced)
        s.step(m)
        ps, vs = s.get_state()
        assert np.array_equal(ps, p) and np.array_equal(vs, v), (config_name, nsplit, m)
        assert np.array_equal(s.get_force()[:, :3], f[:, :3])
    s.set_plan()  # back to the planner's choice, mid-run
    assert s.plan() == nb.force_plan(n)[:2]
    f = _host_steps(p, v, 2, False, lambda t: nb.force(t, 0.01))
    s.step(2)
    ps, vs = s.get_state()
    assert np.array_equal(ps, p) and np.array_equal(vs, v)
    s.close()


def test_set_plan_rejects_the_potential_configuration(cuda):
    s = nb.System(1000, nb.INTEGRATOR_REFERENCE, 0.01, 0.016, 0.95)
    with pytest.raises(nb.NbgbError):
        s.set_plan(nb.force_config_names().index("w8_k2_jt256_s4_pot"), 1)
    s.close()


@pytest.mark.parametrize("config_name", ["w8_k4_jt256_s4_tpair", "w8_k2_jt256_s4_f32x2",
                                         "w8_k2_jt1024_s3_log4"])
def test_kdk64_under_forced_plans(cuda, config_name):
    """FP64 KDK steps write the next j-stream in the plan's layout (paired or
    duplicated sources, log-domain slots): under each forced plan the
    trajectory follows the default plan's to force rounding."""
    n = 3001
    p0, v0, pm, _ = nb.ic_plummer(n, 9)
    m = pm[:, 3].copy()
    out = []
    for cfg in (-1, nb.force_config_names().index(config_name)):
        s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, 0.002, 1.0)
        s.set_plan(cfg, 2 if cfg >= 0 else -1)
        s.set_state64(p0, v0, m)
        s.step(10)
        out.append(s.get_state64())
        s.close()
    dp = np.abs(out[0][0] - out[1][0]).max()
    dv = np.abs(out[0][1] - out[1][1]).max() / np.abs(out[0][1]).max()
    assert dp < 1e-9 and dv < 1e-6, (dp, dv)
