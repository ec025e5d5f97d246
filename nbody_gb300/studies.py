"""Precision study: FP32 forces with compensated sums under an FP64
kick-drift-kick integrator.

    python -m nbody_gb300.studies precision [--n 262144] [--steps 1000]
        [--dt 0.002] [--eps2 1e-4] [--sample 4096] [--every 100] [--seed 262144]

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

from . import (INTEGRATOR_KDK64, System, force_error_stats, force_f64_host, ic_plummer)


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


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision"])
    ap.add_argument("--n", type=int, default=262144)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--dt", type=float, default=0.002)
    ap.add_argument("--eps2", type=float, default=1e-4)
    ap.add_argument("--sample", type=int, default=4096)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--seed", type=int, default=262144)
    a = ap.parse_args(argv)
    r = precision_study(a.n, a.steps, a.dt, a.eps2, a.seed, a.sample, a.every)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
