"""Command-line driver with the reference's flags and stdout format.

    python -m nbody_gb300 [--bodies N] [--iterations N] [--cycle-after N]
        [--seed N] [--no-crosscheck] [--no-cpu] [--gpus N] [--list]
        [--algorithm NAME|INDEX] [--graphics] [--verbose]
        [--softening2 X] [--dt X] [--integrator reference|reference-fused|kdk64]

Mirrors the reference driver's command line (src/nbody.cu:645-701, 749-916)
and per-step line (src/nbody.cu:1024-1053), so tools that parse the
reference's output (scripts/nbody-stats.py) read this one too.  The bodies
are the reference driver's own initial conditions (randomUnitBodies, scale
0.9, velocity scale 8, src/nbody.cu:996), N = --bodies x 1024, softening 0.1
(eps2 0.01), timestep 0.016, damping 0.95 (src/nbody.cu:151-156) unless
overridden.  Two algorithm rows run the device-resident step loop:
GPU_GB300 (the one-sided force kernel) and GPU_GB300_Newton3 (each pair
once); --cycle-after moves to the next row every N steps and an iteration
is one pass through the rows, as in the reference (src/nbody.cu:1055-1068).
The printed milliseconds are the force launch's CUDA-event time, as the
reference prints its algorithm's own timing.  The crosscheck compares each
step's forces with an FP64 all-pairs sum on the host (the reference compares
with its FP32 CPU_SOA) using the reference's relError metric.
"""
from __future__ import annotations

import argparse
import sys
import time

ALGORITHMS = ["GPU_GB300", "GPU_GB300_Newton3"]
FORCE_ALGORITHM = {"GPU_GB300": "onesided", "GPU_GB300_Newton3": "newton3"}


def _gpu_count() -> int:
    try:
        import torch
        return torch.cuda.device_count()
    except Exception:
        return 0


def print_algorithms(n_gpus: int, use_gpus: int, no_cpu: bool) -> None:
    sys.stderr.write("\nAlgorithms available in this build:\n\n")
    for k, name in enumerate(ALGORITHMS):
        suffix = ""
        if n_gpus < 1:
            suffix = " [disabled, no GPUs available]"
        elif use_gpus < 1:
            suffix = " [disabled by user]"
        sys.stdout.write(f"   {k} - {name}{suffix}\n")
    sys.stderr.write("\n")


def parse(argv=None):
    ap = argparse.ArgumentParser(prog="nbody_gb300", add_help=False)
    ap.add_argument("-n", "--bodies", type=int, default=16)
    ap.add_argument("-g", "--gpus", type=int, default=None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-crosscheck", action="store_true")
    ap.add_argument("-i", "--iterations", type=int, default=0)
    ap.add_argument("-c", "--cycle-after", type=int, default=0)
    ap.add_argument("-s", "--seed", type=int, default=7)
    ap.add_argument("-l", "--list", action="store_true")
    ap.add_argument("-a", "--algorithm", default="0")
    ap.add_argument("-G", "--graphics", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("-h", "--help", action="store_true")
    ap.add_argument("--softening2", type=float, default=0.1 * 0.1)
    ap.add_argument("--dt", type=float, default=0.016)
    ap.add_argument("--damping", type=float, default=0.95)
    ap.add_argument("--integrator", choices=["reference", "reference-fused", "kdk64"],
                    default="reference",
                    help="reference: integrateOne, each operation rounded; reference-fused: "
                         "the same with the position update fused, as the reference binary "
                         "built with its own flags computes it; kdk64: FP64 leapfrog")
    return ap.parse_args(argv)


def _check(a) -> str | None:
    if a.bodies < 1:
        return "ERROR: Requested number of bodies less than 1"
    if a.iterations < 0:
        return "ERROR: Requested number of iterations less than 1"
    if a.cycle_after < 0:
        return "ERROR: Requested cycle size less than 1"
    if a.seed < 1:
        return "ERROR: Seed must be nonzero integer value"
    return None


def resolve_algorithm(spec: str) -> int | None:
    try:
        v = int(spec)
        return v if 0 <= v < len(ALGORITHMS) else None
    except ValueError:
        pick = None
        for k, name in enumerate(ALGORITHMS):
            if spec.lower() == name.lower():
                return k
            if name.lower().startswith(spec.lower()):
                pick = k
        return pick


def main(argv=None) -> int:
    a = parse(argv)
    if a.help:
        sys.stderr.write(__doc__)
        return 1
    err = _check(a)
    if err:
        sys.stderr.write(err + "\n")
        return 1
    n_gpus = _gpu_count()
    use_gpus = n_gpus if a.gpus is None else max(0, min(a.gpus, n_gpus))
    if a.graphics:
        sys.stderr.write("Graphics requested, but OpenGL support not compiled in.\n")
    if resolve_algorithm(a.algorithm) is None:
        sys.stderr.write(f"Invalid algorithm '{a.algorithm}'\n")
        print_algorithms(n_gpus, use_gpus, a.no_cpu)
        return 1
    if a.list:
        print_algorithms(n_gpus, use_gpus, a.no_cpu)
        return 0
    if use_gpus < 1:
        sys.stderr.write("ERROR: no GPU available for the GPU_GB300 algorithm\n")
        return 1

    import numpy as np

    import nbody_gb300 as nb

    n = a.bodies * 1024
    crosscheck = not (a.no_crosscheck or a.no_cpu)
    msg = f"Running simulation with {n} particles"
    if crosscheck:
        msg += ", crosscheck enabled"
    msg += ", CPU disabled" if a.no_cpu else ", host FP64 crosscheck"
    msg += f", up to {use_gpus} GPUs"
    sys.stderr.write(msg + "\n")

    pm, vm = nb.ic_reference(n, a.seed)
    integ = {"reference": nb.INTEGRATOR_REFERENCE,
             "reference-fused": nb.INTEGRATOR_REFERENCE_FUSED,
             "kdk64": nb.INTEGRATOR_KDK64}[a.integrator]
    s = nb.System(n, integ, a.softening2, a.dt, a.damping)
    if integ != nb.INTEGRATOR_KDK64:
        s.set_state(pm, vm)
    else:
        s.set_state64(pm[:, :3].astype(np.float64), vm[:, :3].astype(np.float64),
                      pm[:, 3].copy())
    s.set_timing(True)
    width = max(len(x) for x in ALGORITHMS)
    alg = resolve_algorithm(a.algorithm)
    name = ALGORITHMS[alg]
    s.set_force_algorithm(FORCE_ALGORITHM[name])
    steps = iterations = 0
    last = time.monotonic()
    idx = np.arange(n)
    while True:
        p_before = s.get_state()[0] if crosscheck else None
        s.step(1)
        ms = s.last_force_ms()
        rel = None
        if crosscheck:
            f = s.get_force()
            golden = np.zeros_like(f)
            golden[:, :3] = nb.force_f64_host(p_before, a.softening2, idx)[0]
            rel = nb.crosscheck_max_rel_error(f, golden)
        now = time.monotonic()
        if a.verbose or now - last >= 0.1:
            last = now
            sys.stdout.write("\r" + nb.reference_line(name, n, ms, rel, width) + "\n")
            sys.stdout.flush()
        steps += 1
        if a.cycle_after and steps % a.cycle_after == 0:
            steps = 0
            alg += 1
            if alg == len(ALGORITHMS):  # wrapped: one pass through the rows
                alg = 0
                iterations += 1
            name = ALGORITHMS[alg]
            s.set_force_algorithm(FORCE_ALGORITHM[name])
        elif not a.cycle_after:
            iterations += 1
        if a.iterations and iterations >= a.iterations:
            break
    s.close()
    return 0
