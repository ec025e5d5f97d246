"""Studies on the resident GB300 path: the precision study and the batched
ensemble against looping the plain kernel.

    python -m nbody_gb300.studies precision [--n 262144] [--steps 1000]
        [--dt 0.002] [--eps2 1e-4] [--sample 4096] [--every 100] [--seed 262144]
    python -m nbody_gb300.studies batched [--systems 4096] [--steps 100]
        [--dt 0.01] [--eps2 1e-4] [--seed 4096] [--plain-sample 4096]
    python -m nbody_gb300.studies forms [--n 262144] [--sample 4096]

Forms study: the force of one configuration whose pairs all use rsqrt and of
one that takes every fourth source pair in the log domain, on a seeded
Plummer sphere and on a 16,384-body uniform ball (m = 1/N), each against the
FP64 all-pairs sum on a seeded subsample (the whole ball), with the time per
evaluation.

Precision study:

Seeded Plummer sphere (G = M = a = 1, equal masses), state resident on the
GPU.  Reports the max and RMS per-body relative force error of the GPU's FP32
forces against the library's FP64 all-pairs sum (nbgb_force_f64_host) on a
seeded subsample of targets, at the start and at the end, and the relative
total-energy drift |E(t) - E(0)| / |E(0)| with E from the FP64 reductions
(nbgb_system_diagnostics), sampled every `every` steps.  Prints one JSON
object.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import (INTEGRATOR_KDK64, System, force, force_config_names, force_error_stats,
               force_f64_host, ic_plummer, ic_uniform_ball)


def precision_study(n: int = 262144, steps: int = 1000, dt: float = 0.002, eps2: float = 1e-4,
                    seed: int = 262144, n_sample: int = 4096, every: int = 100) -> dict:
    import torch

    p3, v3, pm, _ = ic_plummer(n, seed)
    mass = pm[:, 3].copy()
    sysm = System(n, INTEGRATOR_KDK64, eps2, dt, 1.0)
    sysm.set_state64(p3, v3, mass)
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, min(n_sample, n), replace=False))

    d0 = sysm.diagnostics()
    e0 = d0["energy"]

    # force error at t = 0 (the planner gives the same kernel plan as the
    # system's own first force pass on these positions)
    from . import force as gpu_force
    f_start = gpu_force(torch.from_numpy(pm).cuda(), eps2).cpu().numpy()
    t64 = time.perf_counter()
    f64, _ = force_f64_host(pm, eps2, idx)
    host_s = time.perf_counter() - t64
    err_start = force_error_stats(f_start, f64, idx)

    energies = [(0, e0)]
    step_s = 0.0
    done = 0
    while done < steps:
        k = min(every, steps - done)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sysm.step(k)
        sysm.synchronize()
        step_s += time.perf_counter() - t0
        done += k
        energies.append((done, sysm.diagnostics()["energy"]))

    pm_end, _ = sysm.get_state()
    f_end = sysm.get_force()
    f64_end, _ = force_f64_host(pm_end, eps2, idx)
    err_end = force_error_stats(f_end, f64_end, idx)
    d1 = sysm.diagnostics()
    sysm.close()

    drift = [abs(e - e0) / abs(e0) for _, e in energies]
    return {
        "study": "precision",
        "n_bodies": n, "steps": steps, "dt": dt, "softeningSquared": eps2, "seed": seed,
        "integrator": "FP64 kick-drift-kick, FP32 forces with TwoSum across tiles",
        "force_error_start": {"max": err_start[0], "rms": err_start[1], "sample": int(len(idx))},
        "force_error_end": {"max": err_end[0], "rms": err_end[1], "sample": int(len(idx))},
        "energy_start": e0, "energy_end": d1["energy"],
        "energy_drift_final": drift[-1], "energy_drift_max": max(drift),
        "energy_samples": [[s, e] for s, e in energies],
        "momentum_end": d1["momentum"].tolist(),
        "angular_momentum_start": d0["angular_momentum"].tolist(),
        "angular_momentum_end": d1["angular_momentum"].tolist(),
        "seconds_in_steps": step_s,
        "ms_per_step": 1e3 * step_s / max(steps, 1),
        "interactions_per_s": float(n) * n * steps / step_s if step_s > 0 else None,
        "fp64_check_seconds": host_s,
    }


def ensemble_systems(n_systems: int, n_lo: int, n_hi: int, seed: int, mass_lo: float = 0.5,
                     mass_hi: float = 1.5):
    """Seeded systems: N log-uniform in [n_lo, n_hi], uniform ball of radius 1,
    masses U[mass_lo, mass_hi] / N, zero velocities."""
    from . import ic_uniform_ball
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(n_lo), np.log(n_hi), n_systems))
    sizes = np.clip(np.rint(sizes).astype(int), n_lo, n_hi)
    out = []
    for k, n in enumerate(sizes):
        pm, _ = ic_uniform_ball(int(n), seed * 100003 + k, 1.0, mass_lo, mass_hi)
        p = pm[:, :3].astype(np.float64)
        out.append((p, np.zeros_like(p), pm[:, 3].copy()))
    return out


def batched_study(n_systems: int = 4096, n_lo: int = 64, n_hi: int = 8192, steps: int = 100,
                  dt: float = 0.01, eps2: float = 1e-4, seed: int = 4096,
                  plain_sample: int = 4096, plain_graphs: bool = True) -> dict:
    """Every system advanced `steps` FP64 KDK steps, once through the ensemble
    (one persistent force launch per step for all systems, CUDA-graph ticks)
    and once by looping the plain single-system path over the systems (one
    System per system, stepped as a user of that path would: its step body
    captured once into a CUDA graph and replayed, the graph's capture and
    instantiation inside the timed region; plain_graphs=False launches
    eagerly instead).  The plain loop may run on a seeded subsample of
    `plain_sample` systems; its systems/s then scales by the sample's share
    of the interactions (stated in the result)."""
    import torch

    from . import INTEGRATOR_KDK64, Ensemble, System

    systems = ensemble_systems(n_systems, n_lo, n_hi, seed)
    sizes = np.array([p.shape[0] for p, _, _ in systems])
    inter = float((sizes.astype(np.float64) ** 2).sum()) * (steps + 1)

    e = Ensemble(int(sizes.sum()), n_systems, eps2)
    t0 = time.perf_counter()
    slots = [e.add(p, v, m, dt, steps) for p, v, m in systems]
    admit_s = time.perf_counter() - t0
    assert all(s is not None for s in slots)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.tick(steps + 1)
    e.synchronize()
    ens_s = time.perf_counter() - t0
    assert len(e.finished()) == n_systems
    e.close()

    # plain loop (sequential, one system at a time)
    rng = np.random.default_rng(seed + 1)
    pick = np.arange(n_systems) if plain_sample >= n_systems else np.sort(
        rng.choice(n_systems, plain_sample, replace=False))
    plain_s = 0.0
    plain_inter = 0.0
    for k in pick:
        p, v, m = systems[k]
        n = p.shape[0]
        s = System(n, INTEGRATOR_KDK64, eps2, dt, 1.0)
        s.use_graph(plain_graphs)
        s.set_state64(p, v, m)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(steps)
        s.synchronize()
        plain_s += time.perf_counter() - t0
        plain_inter += float(n) * n * (steps + 1)
        s.close()
    plain_full_s = plain_s * inter / plain_inter
    return {
        "study": "batched",
        "systems": n_systems, "n_range": [n_lo, n_hi], "steps": steps, "dt": dt,
        "softeningSquared": eps2, "seed": seed, "total_bodies": int(sizes.sum()),
        "interactions": inter,
        "ensemble_seconds": ens_s, "ensemble_systems_per_s": n_systems / ens_s,
        "ensemble_interactions_per_s": inter / ens_s,
        "ensemble_admission_seconds": admit_s,
        "plain_sample": int(len(pick)), "plain_seconds_sample": plain_s,
        "plain_seconds_full_estimate": plain_full_s,
        "plain_systems_per_s": n_systems / plain_full_s,
        "plain_interactions_per_s": plain_inter / plain_s,
        "plain_mode": "CUDA graph per system" if plain_graphs else "eager launches",
        "speedup": plain_full_s / ens_s,
    }


def forms_study(n: int = 262144, sample: int = 4096, eps2: float = 1e-4,
                configs=(25, 27)) -> dict:
    import torch
    names = force_config_names()
    _, _, pm_plummer, _ = ic_plummer(n, 3)
    pm_ball, _ = ic_uniform_ball(16384, 16384)
    out = {}
    for case, pm_np, k in (("plummer", pm_plummer, min(sample, n)), ("ball16384", pm_ball, 16384)):
        m = pm_np.shape[0]
        idx = (np.arange(m) if k >= m else
               np.sort(np.random.default_rng(7).choice(m, k, replace=False)))
        ref, _ = force_f64_host(pm_np, eps2, idx)
        pm = torch.from_numpy(pm_np).cuda()
        rows = {}
        for c in configs:
            f = force(pm, eps2, config=c)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                force(pm, eps2, out=f, config=c)
            e1.record()
            torch.cuda.synchronize()
            mx, rms = force_error_stats(f.cpu().numpy(), ref, idx)
            rows[names[c]] = {"max_rel_err_vs_fp64": mx, "rms_rel_err_vs_fp64": rms,
                              "ms": e0.elapsed_time(e1) / 3}
        out[case] = {"n": m, "targets_checked": len(idx), "configs": rows}
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="study", required=True)
    pr = sub.add_parser("precision")
    pr.add_argument("--n", type=int, default=262144)
    pr.add_argument("--steps", type=int, default=1000)
    pr.add_argument("--dt", type=float, default=0.002)
    pr.add_argument("--eps2", type=float, default=1e-4)
    pr.add_argument("--sample", type=int, default=4096)
    pr.add_argument("--every", type=int, default=100)
    pr.add_argument("--seed", type=int, default=262144)
    ba = sub.add_parser("batched")
    ba.add_argument("--systems", type=int, default=4096)
    ba.add_argument("--n-lo", type=int, default=64)
    ba.add_argument("--n-hi", type=int, default=8192)
    ba.add_argument("--steps", type=int, default=100)
    ba.add_argument("--dt", type=float, default=0.01)
    ba.add_argument("--eps2", type=float, default=1e-4)
    ba.add_argument("--seed", type=int, default=4096)
    ba.add_argument("--plain-sample", type=int, default=4096)
    ba.add_argument("--plain-eager", action="store_true",
                    help="loop the plain path with eager launches instead of CUDA graphs")
    fo = sub.add_parser("forms")
    fo.add_argument("--n", type=int, default=262144)
    fo.add_argument("--sample", type=int, default=4096)
    a = ap.parse_args(argv)
    if a.study == "forms":
        r = forms_study(a.n, a.sample)
    elif a.study == "precision":
        r = precision_study(a.n, a.steps, a.dt, a.eps2, a.seed, a.sample, a.every)
    else:
        r = batched_study(a.systems, a.n_lo, a.n_hi, a.steps, a.dt, a.eps2, a.seed,
                          a.plain_sample, not a.plain_eager)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
