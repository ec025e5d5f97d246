"""Ensembles: one persistent force launch over many systems of uneven N.
Forces against FP64, alone-vs-mixed bit identity (also when systems join and
leave mid-run), admission limits, and agreement with the single-system path."""
import numpy as np
import pytest

from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

TOL_VS_FP64 = 5e-6
EPS2 = 1e-4


def _ball(n, seed):
    pm, _ = nb.ic_uniform_ball(n, seed, 1.0, 0.5, 1.5)
    p = pm[:, :3].astype(np.float64)
    v = np.zeros_like(p)
    return p, v, pm[:, 3].copy(), pm


def _f64(pm):
    f = np.zeros((pm.shape[0], 4))
    f[:, :3] = O.ieee().forces_f64(pm, float(np.float32(EPS2)))
    return f


@pytest.mark.parametrize("variant,jt,nsplit", [(0, 128, 1), (1, 256, 1), (1, 512, 3),
                                               (0, 1024, 2), (1, 1024, 1), (-1, 256, 1),
                                               (0, 16, 1), (3, 32, 2)])
def test_initial_forces_match_fp64(cuda, variant, jt, nsplit):
    e = nb.Ensemble(60000, 16, EPS2)
    for b in range(32):
        e.set_bucket_plan(b, variant, jt, nsplit)
    sizes = [1, 33, 64, 700, 1000, 2500, 5003, 8192]
    slots, pms = [], []
    for k, n in enumerate(sizes):
        p, v, m, pm = _ball(n, 100 + k)
        slots.append(e.add(p, v, m, 0.01, 5))
        pms.append(pm)
    e.tick(1)  # initial accelerations only
    e.synchronize()
    for s, pm in zip(slots, pms):
        p1, v1, a = e.get_state(s)
        assert np.array_equal(p1, pm[:, :3].astype(np.float64))  # nothing moved yet
        if pm.shape[0] == 1:
            assert np.all(a[0, :3] == 0)
            continue
        assert O.per_body_rel_error(a, _f64(pm))[0] <= TOL_VS_FP64
    e.close()


def test_alone_and_mixed_are_bit_identical_with_joins_and_leaves(cuda):
    dt, steps = 0.002, 6
    cases = {n: _ball(n, n) for n in (300, 1500, 4100, 7000)}

    def run(members, join_at):
        e = nb.Ensemble(40000, 8, EPS2)
        slots, out, t = {}, {}, 0
        pending = sorted(members, key=lambda n: join_at.get(n, 0))
        while pending or slots:
            for n in list(pending):
                if join_at.get(n, 0) <= t:
                    p, v, m, _ = cases[n]
                    slots[n] = e.add(p, v, m, dt, steps)
                    pending.remove(n)
            e.tick(1)
            t += 1
            for s in e.finished():
                n = next(k for k, v in slots.items() if v == s)
                out[n] = e.get_state(s)
                e.remove(s)
                del slots[n]
        e.close()
        return out

    alone = {n: run([n], {})[n] for n in cases}
    mixed = run(list(cases), {300: 0, 1500: 2, 4100: 3, 7000: 9})
    for n in cases:
        for a, b in zip(alone[n], mixed[n]):
            assert np.array_equal(a, b), n


def test_matches_single_system_kdk(cuda):
    n, dt, steps = 3000, 0.002, 20
    p, v, pm, _ = nb.ic_plummer(n, 31)
    m = pm[:, 3].copy()
    s = nb.System(n, nb.INTEGRATOR_KDK64, EPS2, dt, 1.0)
    s.set_state64(p, v, m)
    s.step(steps)
    ps, vs = s.get_state64()
    s.close()
    e = nb.Ensemble(n, 1, EPS2)
    slot = e.add(p, v, m, dt, steps)
    e.tick(steps + 1)
    e.synchronize()
    assert e.finished() == [slot]
    pe, ve, _ = e.get_state(slot)
    e.close()
    # different kernel plans round differently (the single-system plan takes
    # every fourth source pair in the log domain, whose per-term error is a
    # few times the rsqrt form's); after 20 smooth steps the states agree to
    # small multiples of the FP32 force error times dt
    assert np.abs(pe - ps).max() <= 1e-9 * np.abs(ps).max()
    assert np.abs(ve - vs).max() <= 5e-8 * np.abs(vs).max()


def test_admission_limits_and_reuse(cuda):
    e = nb.Ensemble(5000, 3, EPS2)
    p, v, m, _ = _ball(2000, 1)
    a = e.add(p, v, m, 0.01, 2)
    b = e.add(p, v, m, 0.01, 2)
    assert a is not None and b is not None
    assert e.add(p, v, m, 0.01, 2) is None  # bodies exhausted
    q, w, mm, _ = _ball(500, 2)
    c = e.add(q, w, mm, 0.01, 1)
    assert c is not None
    assert e.add(q, w, mm, 0.01, 1) is None  # slots exhausted
    e.tick(3)
    e.synchronize()
    assert sorted(e.finished()) == sorted([a, b, c])
    e.remove(a)
    assert e.add(p, v, m, 0.01, 1) is not None  # space reused
    assert e.active() == 3
    e.close()


def test_energy_conserved_in_ensemble(cuda):
    n = 2048
    p, v, pm, _ = nb.ic_plummer(n, 44)
    m = pm[:, 3].copy()
    e = nb.Ensemble(3 * n, 3, EPS2)
    slot = e.add(p, v, m, 0.002, 200)
    e.tick(201)
    e.synchronize()
    p1, v1, _ = e.get_state(slot)
    e.close()

    def energy(pos, vel):
        pm4 = np.zeros((n, 4), np.float32)
        pm4[:, :3] = pos
        pm4[:, 3] = m
        phi = O.ieee().potential_f64(pm4, float(np.float32(EPS2)))
        return 0.5 * (m * (vel ** 2).sum(1)).sum() + 0.5 * (m * phi).sum()

    e0, e1 = energy(p, v), energy(p1, v1)
    assert abs(e1 - e0) / abs(e0) < 1e-4


def test_signed_masses_use_rsqrt_pairs(cuda):
    """A system with a negative mass has no log2 masses: the ensemble keeps it
    on rsqrt-only pairs (no status bit, finite forces), and its first forces
    match FP64 like any other system's; its neighbours keep log-domain pairs."""
    e = nb.Ensemble(20000, 4, EPS2)
    p, v, m, pm = _ball(3000, 71)
    m = m.copy()
    m[0] = -m[0]
    m[1500] = -0.5 * m[1500]
    pm = pm.copy()
    pm[:, 3] = m
    p2, v2, m2, pm2 = _ball(2000, 72)
    a_slot = e.add(p, v, m, 0.01, 3)
    b_slot = e.add(p2, v2, m2, 0.01, 3)
    e.tick(1)
    e.synchronize()
    assert nb.last_status() == 0
    for slot, ref_pm in ((a_slot, pm), (b_slot, pm2)):
        _, _, a = e.get_state(slot)
        assert np.all(np.isfinite(a))
        assert O.per_body_rel_error(a, _f64(ref_pm))[0] <= TOL_VS_FP64
    e.close()


def test_substeps_give_identical_results_and_fewer_ticks(cuda):
    """Sub-cycling: a system taking `sub` steps per tick does exactly the
    same KDK steps, so its final state is bit-identical to the one-step-per-
    tick run alone, whatever the mix; it finishes after 1 + ceil(steps/sub)
    ticks."""
    dt = 0.002
    cases = [(300, 13, 4), (1500, 9, 8), (4100, 7, 1), (700, 10, 3)]  # n, steps, sub

    def alone(n, steps):
        p, v, m, _ = _ball(n, n)
        e = nb.Ensemble(10000, 2, EPS2)
        s = e.add(p, v, m, dt, steps)
        e.tick(steps + 1)
        e.synchronize()
        assert e.finished() == [s]
        out = e.get_state(s)
        e.close()
        return out

    ref = {n: alone(n, steps) for n, steps, _ in cases}
    e = nb.Ensemble(40000, 8, EPS2)
    slots = {}
    for n, steps, sub in cases:
        p, v, m, _ = _ball(n, n)
        slots[n] = e.add(p, v, m, dt, steps)
        e.set_substeps(slots[n], sub)
    done_at, t = {}, 0
    while len(done_at) < len(cases) and t < 50:
        e.tick(1)
        t += 1
        for s in e.finished():
            n = next(k for k, v in slots.items() if v == s)
            if n not in done_at:
                done_at[n] = t
                got = e.get_state(s)
                for a, b in zip(got, ref[n]):
                    assert np.array_equal(a, b), n
                e.remove(s)
    e.close()
    for n, steps, sub in cases:
        assert done_at[n] == 1 + -(-steps // sub), (n, done_at[n])


def test_newton3_systems_in_the_ensemble(cuda):
    """Systems at or above the Newton-3 threshold are evaluated with the
    Newton's-third-law kernel beside work-queue systems: their first forces
    match FP64 like the others, and 20 KDK steps agree with the
    single-system Newton-3 path to FP64-order rounding."""
    e = nb.Ensemble(40000, 8, EPS2)
    e.set_newton3_min(4096)
    sizes = [3000, 5000, 9000, 2100, 4096]
    slots, pms = {}, {}
    for n in sizes:
        p, v, m, pm = _ball(n, 300 + n)
        slots[n] = e.add(p, v, m, 0.002, 20)
        pms[n] = pm
    e.tick(1)  # initial accelerations only
    e.synchronize()
    assert nb.last_status() == 0
    for n in sizes:
        _, _, a = e.get_state(slots[n])
        assert O.per_body_rel_error(a, _f64(pms[n]))[0] <= TOL_VS_FP64, n
    e.tick(20)
    e.synchronize()
    assert sorted(e.finished()) == sorted(slots.values())
    for n in (5000, 9000):
        pe, ve, _ = e.get_state(slots[n])
        p, v, m, _ = _ball(n, 300 + n)
        s = nb.System(n, nb.INTEGRATOR_KDK64, EPS2, 0.002, 1.0)
        s.set_force_algorithm("newton3")
        s.set_state64(p, v, m)
        s.step(20)
        ps, vs = s.get_state64()
        s.close()
        assert np.abs(pe - ps).max() <= 1e-9 * np.abs(ps).max(), n
        # v starts at 0 and is the sum of 20 dt-weighted FP32 forces, whose
        # FP64 summation order may differ by an FP32 ulp between the runs
        _, _, a = e.get_state(slots[n])
        bound = 4 * 20 * 0.002 * np.abs(a[:, :3]).max() * 2.0 ** -23
        assert np.abs(ve - vs).max() <= bound, n
    e.close()
