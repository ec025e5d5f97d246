"""Generate tests/golden/*.npz from the reference's own CPU objects.

Run in a container where the reference sources are present:

    make -C oracle all ref REF=<reference checkout>   # oracle/_ref/libnbody_ref.so
    python tests/golden/gen_golden.py

    python tests/golden/gen_golden.py c1_ball16384     # only the named fixtures

Each fixture stores its inputs next to the outputs, so the tests need neither
the reference nor this script.  Forces come from the reference's compiled
ComputeGravitation_AOS / ComputeGravitation_SOA (src/nbody_CPU_AOS.cpp:51-98,
src/nbody_CPU_SOA.cpp:53-105, built with the reference's flags by
oracle/Makefile); reference-style initial conditions come from its compiled
seedRandom/randomUnitBodies (src/nbody_util.cpp:81-144).  The FP64 forces are
the oracle's own all-pairs sum.  Trajectories apply the reference's integrator
formula (src/nbody.cu:158-182, restated in oracle/nbody_oracle.c) to the
reference's forces; the 16,384-body case uses the reference driver's own
compiled integrator instead (oracle/ref_shim.cpp exports the static
integrateGravitation_SOA).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402


def uniform_ball(n: int, seed: int, radius: float = 1.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 3), np.float64)
    k = 0
    while k < n:
        p = rng.uniform(-1.0, 1.0, (2 * n, 3))
        p = p[(p * p).sum(1) <= 1.0]
        m = min(n - k, len(p))
        out[k:k + m] = p[:m]
        k += m
    return (out * radius).astype(np.float32)


def plummer(n: int, seed: int) -> np.ndarray:
    """Plummer sphere positions (a=1, M=1), Aarseth-Henon-Wielen radii."""
    rng = np.random.default_rng(seed)
    x1 = rng.uniform(1e-10, 0.999, n)
    r = 1.0 / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
    u = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - u * u)
    pm = np.zeros((n, 4), np.float32)
    pm[:, 0] = r * s * np.cos(ph)
    pm[:, 1] = r * s * np.sin(ph)
    pm[:, 2] = r * u
    pm[:, 3] = 1.0 / n
    return pm


def f64_as4(pm, eps2):
    # the FP32 paths see eps2 rounded to binary32; the FP64 sum uses that value
    f = O.ieee().forces_f64(pm, float(np.float32(eps2)))
    out = np.zeros((pm.shape[0], 4), np.float64)
    out[:, :3] = f
    return out


def main() -> None:
    assert O.ref_available(), "build oracle/_ref first: make -C oracle all ref"
    R = O.ref()
    out = {}

    # 1. unit ball, m = 1/N, eps2 = 1e-4 (the 16K-body plain case, scaled down)
    n = 2048
    pm = np.zeros((n, 4), np.float32)
    pm[:, :3] = uniform_ball(n, 101)
    pm[:, 3] = 1.0 / n
    out["ball2048"] = dict(posMass=pm, eps2=np.float32(1e-4),
                           force_aos=R.forces_aos(pm, 1e-4),
                           force_soa=R.forces_soa(pm, 1e-4),
                           force_f64=f64_as4(pm, 1e-4))

    # 2. the reference driver's own initial conditions (seed 7, 1024 bodies,
    #    softening 0.1 -> eps2 0.01), src/nbody.cu:80-81,151-156,996
    pos, vel = R.random_unit_bodies(1024, 7, 0.9, 8.0)
    out["refic1024_seed7"] = dict(posMass=pos, velInvMass=vel, eps2=np.float32(0.01),
                                  force_aos=R.forces_aos(pos, 0.01),
                                  force_f64=f64_as4(pos, 0.01))

    # 3. Plummer sphere, 4096 bodies (centrally concentrated)
    pm = plummer(4096, 202)
    out["plummer4096"] = dict(posMass=pm, eps2=np.float32(1e-4),
                              force_aos=R.forces_aos(pm, 1e-4),
                              force_f64=f64_as4(pm, 1e-4))

    # 4. ragged N: 1000 bodies padded with zero-mass bodies to 1024 for the
    #    reference (its loops assume N % 1024 == 0, src/nbody_CPU_AOS.cpp:58-59)
    n = 1000
    pm = np.zeros((1024, 4), np.float32)
    pm[:n, :3] = uniform_ball(n, 303)
    rng = np.random.default_rng(304)
    pm[:n, 3] = rng.uniform(0.5, 1.5, n).astype(np.float32) / n
    fa = R.forces_aos(pm, 1e-4)
    out["ragged1000"] = dict(posMass=pm[:n].copy(), eps2=np.float32(1e-4),
                             force_aos=fa[:n].copy(),
                             force_f64=f64_as4(pm[:n].copy(), 1e-4))

    # 5. 10-step trajectory of the plain case (1024 bodies, dt 0.01, damping
    #    0.95, v0 = 0, invMass = 1/m), positions kept after steps 1, 5, 10
    n = 1024
    pm = np.zeros((n, 4), np.float32)
    pm[:, :3] = uniform_ball(n, 404)
    pm[:, 3] = 1.0 / n
    vel = np.zeros((n, 4), np.float32)
    vel[:, 3] = 1.0 / pm[:, 3]
    traj = dict(posMass0=pm.copy(), velInvMass0=vel.copy(), eps2=np.float32(1e-4),
                dt=np.float32(0.01), damping=np.float32(0.95))
    p, v = pm.copy(), vel.copy()
    for step in range(1, 11):
        f = R.forces_aos(p, 1e-4)
        if step == 1:
            traj["force_step1"] = f.copy()
        O.ieee().integrate(p, v, f, 0.01, 0.95)
        if step in (1, 5, 10):
            traj[f"posMass{step}"] = p.copy()
            traj[f"velInvMass{step}"] = v.copy()
    out["traj1024"] = traj

    # 6. the plain single-system configuration exactly: N = 16,384 uniform in
    #    the unit ball, m = 1/N, v = 0, eps2 = 1e-4, dt = 0.01, 10 steps with
    #    the reference driver's own compiled integrator (integrateGravitation_SOA
    #    through oracle/ref_shim.cpp, damping 0.95 = the driver's default,
    #    src/nbody.cu:152) on the reference's CPU_AOS forces
    if O.ref_driver_available():
        n = 16384
        pm = np.zeros((n, 4), np.float32)
        pm[:, :3] = uniform_ball(n, 505)
        pm[:, 3] = np.float32(1.0 / n)
        vel = np.zeros((n, 4), np.float32)
        vel[:, 3] = 1.0 / pm[:, 3]
        c1 = dict(posMass0=pm.copy(), velInvMass0=vel.copy(), eps2=np.float32(1e-4),
                  dt=np.float32(0.01), damping=np.float32(0.95))
        p, v = pm.copy(), vel.copy()
        for step in range(1, 11):
            f = R.forces_aos(p, 1e-4)
            if step == 1:
                c1["force_aos0"] = f.copy()
            O.ref_driver().integrate(p, v, f, 0.01, 0.95)
            if step in (1, 10):
                c1[f"posMass{step}"] = p.copy()
                c1[f"velInvMass{step}"] = v.copy()
        out["c1_ball16384"] = c1

    # 7. the plain large system's input (N = 1,048,576 Plummer, the bench's
    #    seed), forces of the reference's compiled CPU_AOS on every body, kept
    #    for a seeded 1,024-body sample (the bench's accuracy sample) with
    #    their FP64 sums; the input itself is regenerated by the tests from
    #    its seed (oracle restatement of the library's Plummer generator) and
    #    checked against the stored checksum
    if os.environ.get("NBODY_GOLDEN_LARGE") or "c2_plummer1m_sample" in sys.argv[1:]:
        import hashlib
        n, seed = 1 << 20, 20260
        _, _, pm = O.ieee().ic_plummer(n, seed)
        idx = np.random.default_rng(7).choice(n, 1024, replace=False)
        fa = R.forces_aos(pm, 1e-4)
        out["c2_plummer1m_sample"] = dict(
            n=np.int64(n), seed=np.int64(seed), eps2=np.float32(1e-4), idx=idx.astype(np.int64),
            posMass_sha256=np.bytes_(hashlib.sha256(pm.tobytes()).hexdigest().encode()),
            posMass_idx=pm[idx].copy(), force_aos=fa[idx].copy(),
            force_f64=O.ieee().forces_f64(pm, float(np.float32(1e-4)), idx))

    only = set(sys.argv[1:])
    for name, d in out.items():
        if only and name not in only:
            continue
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **d)
        print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
