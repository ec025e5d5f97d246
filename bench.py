"""Headline benchmark: all-pairs gravity on one GB300, interactions/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step" = one force evaluation + one integrate step): the plain
large system, N = 1,048,576 bodies of a seeded Plummer sphere (G = M = a = 1,
equal masses), FP32 posMass, softeningSquared = 1e-4, dt = 0.005, FP64
kick-drift-kick integrator, state resident in HBM.  Metric: 10^9
interactions/s with N^2 interactions per force evaluation (self pairs
included, the reference's convention, src/nbody.cu:1026) and 20 FLOP per
interaction (src/nbody.cu:1027).

  value     device-timed: sum of per-step CUDA-event times on the system's
            stream, L2 flushed (256 MiB write) between steps outside the events
  e2e       the reference-facing drop-in ComputeGravitation_GPU_GB300 with
            HOST buffers: per step pinned H2D of posMass, the call, D2H of the
            forces, all inside a host-clock timed region
  roofline  the force kernel: 20 N^2 FLOP / its CUDA-event launch time, over
            the FP32 pipe peak measured by the library's FMA microbenchmark
            on this GPU (max of scalar and f32x2), plus the MUFU ceiling
  cpu_baseline  the oracle's restatement of the reference's CPU_SOA loop
            (OpenMP, all host threads) on a bounded sample of target bodies
            against all N sources

--impl reference times the reference's CPU implementation of the path (the
reference's own compiled CPU_SOA when oracle/_ref was built on this machine,
else the oracle's restatement of it) on the same workload, each step a
bounded sample of targets.  Multi-GPU runs are independent replicas (the
path needs no exchange on one node of replicas); value sums all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_BODIES = 1 << 20
EPS2 = 1e-4
DT = 0.005
SEED = 20260
FLOP = 20
METRIC = "G interactions/s (20 FLOP/interaction)"
UNIT = "1e9 interactions/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def _barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def _allmax(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _allsum(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate(ws: int, seconds: float, interactions: float):
    """Whole-job rate of independent replicas: every rank's interactions
    over the slowest rank's time (1e9 interactions/s), and that time."""
    t_max = _allmax(ws, seconds)
    total = _allsum(ws, interactions)
    return total / t_max / 1e9, t_max, total


# ---------------------------------------------------------------------------
# nvidia-smi clock sampling during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        smax = max(r[1] for r in rows)
        load = [r for r in rows if r[0] > 0.5 * smax] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[2][k] == "Active"})
        return {"sm_mhz": float(np.median([r[0] for r in load])), "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU measurement (oracle restatement of CPU_SOA, or the reference's own)
# ---------------------------------------------------------------------------
def cpu_rate(pm: np.ndarray, seconds: float):
    """Time the CPU_SOA loop over a contiguous sample of targets against all N
    sources, sized to take about `seconds`.  Returns (rate 1e9/s, s, info)."""
    from oracle import oracle as O
    O.build(ref=False)
    n = pm.shape[0]
    impl = O.fast()
    run = impl.soa_timer(pm, EPS2)
    # calibrate on a small slice
    t0 = time.perf_counter()
    run(0, 64)
    dt = max(time.perf_counter() - t0, 1e-6)
    per_target = dt / 64
    ni = int(min(n, max(256, seconds / per_target)))
    ni = (ni // 64) * 64 or 64
    t0 = time.perf_counter()
    run(0, ni)
    el = time.perf_counter() - t0
    rate = ni * float(n) / el / 1e9
    info = {"kind": "port", "cores": impl.num_threads(),
            "sample": f"{ni} target bodies x {n} sources of the same Plummer system "
                      f"({ni * n:.3e} interactions, {el:.1f} s), oracle restatement of "
                      "CPU_SOA (src/nbody_CPU_SOA.cpp:53-105) built with the reference's "
                      "flags (-O3 -ffast-math -fopenmp)"}
    return rate, el, info


def profiled_traffic(config_name: str, n: int, nsplit: int):
    """DRAM bytes per force launch from the committed ncu summary, when it was
    captured for this kernel configuration, N and j-split (else None)."""
    path = os.path.join(ROOT, "profiles", "force_kernel_n1048576_dram.md")
    if not os.path.exists(path):
        return None
    import re
    for line in open(path):
        m = re.match(r"traffic_bytes_per_launch:\s*(\d+)\s+config\s+(\S+)\s+n\s+(\d+)"
                     r"\s+nsplit\s+(\d+)", line.strip())
        if m and m.group(2) == config_name and int(m.group(3)) == n and \
                int(m.group(4)) == nsplit:
            return int(m.group(1))
    return None


def run_reference_arm(args, ws, rank):
    if rank != 0:
        return
    import nbody_gb300 as nb
    from oracle import oracle as O
    O.build(ref=False)
    _, _, pm, _ = nb.ic_plummer(N_BODIES, SEED)
    impl = O.fast()
    run = impl.soa_timer(pm, EPS2)
    t0 = time.perf_counter()
    run(0, 64)
    per_target = max(time.perf_counter() - t0, 1e-6) / 64
    per_step_s = 8.0
    ni = int(min(N_BODIES, max(256, per_step_s / per_target))) // 64 * 64
    for _ in range(args.warmup):
        run(0, min(ni, 256))
    times = []
    for k in range(args.steps):
        lo = (k * ni) % max(1, N_BODIES - ni)
        t0 = time.perf_counter()
        run(lo, lo + ni)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    rate = ni * float(N_BODIES) * args.steps / tot / 1e9
    ms_full = N_BODIES * float(N_BODIES) / (rate * 1e9) * 1e3
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_full,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer sphere)",
        "config": {"workload": "plain large system: N=1,048,576 Plummer, FP32, eps2=1e-4",
                   "n_bodies": N_BODIES, "sample_targets_per_step": ni,
                   "l2": "host CPU run; no GPU"},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": impl.num_threads(),
                         "kind": "port",
                         "sample": f"{ni} targets x {N_BODIES} sources per step "
                                   f"({ni * N_BODIES:.3e} interactions), oracle restatement "
                                   "of the reference's CPU_SOA with its build flags (the "
                                   "reference's own CPU objects are built only where its "
                                   "sources are present; tests check the restatement "
                                   "against them)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
def run_gb300(args, ws, rank, local):
    import torch

    import nbody_gb300 as nb
    from nbody_gb300 import build as B
    B.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # pipe peaks on this GPU
    ffma, _ = nb.measure_peak("ffma")
    ffma2, _ = nb.measure_peak("ffma2")
    mufu, _ = nb.measure_peak("mufu")
    fp32_peak = max(ffma, ffma2)

    n = args.n
    p3, v3, pm_np, _ = nb.ic_plummer(n, SEED + rank)
    sysm = nb.System(n, nb.INTEGRATOR_KDK64, EPS2, DT, 1.0)
    sysm.set_state64(p3, v3, pm_np[:, 3].copy())
    if args.force == "newton3":
        sysm.set_force_algorithm("newton3")
    sysm.set_timing(True)
    stream = torch.cuda.ExternalStream(sysm.stream, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    for _ in range(args.warmup):
        sysm.step(1)
    sysm.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    force_ms = []
    clocks = Clocks(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
                    if os.environ.get("CUDA_VISIBLE_DEVICES", "").isdigit() else local)
    _barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # evict L2 between steps (outside the events)
            ev[k][0].record(stream)
        sysm.step(1)
        ev[k][1].record(stream)
        force_ms.append(sysm.last_force_ms())
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    _barrier(ws)
    sysm.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_dev = sum(step_ms) / 1e3
    inter = float(n) * float(n) * args.steps
    value, t_max, total_inter = aggregate(ws, t_dev, inter)
    kernel_ms = float(np.mean(force_ms))
    achieved = FLOP * float(n) * float(n) / (kernel_ms * 1e-3)
    cfg, nsplit = sysm.plan()
    cfg_name = nb.force_config_names()[cfg] if args.force == 'onesided' else 'newton3'
    traffic = profiled_traffic(cfg_name, n, nsplit)
    sysm.close()

    # e2e: the drop-in entry point with host buffers
    pm_h = torch.from_numpy(pm_np).pin_memory()
    f_h = torch.empty((n, 4), dtype=torch.float32).pin_memory()
    pm_d = torch.empty((n, 4), dtype=torch.float32, device=dev)
    f_d = torch.empty((n, 4), dtype=torch.float32, device=dev)
    for _ in range(max(1, args.warmup)):
        pm_d.copy_(pm_h, non_blocking=True)
        nb.ComputeGravitation_GPU_GB300(f_d, pm_d, EPS2, n)
        f_h.copy_(f_d, non_blocking=True)
        torch.cuda.synchronize()
    _barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ms_calls = []
    for _ in range(args.steps):
        pm_d.copy_(pm_h, non_blocking=True)
        ms_calls.append(nb.ComputeGravitation_GPU_GB300(f_d, pm_d, EPS2, n))
        f_h.copy_(f_d, non_blocking=True)
        torch.cuda.synchronize()
    e2e_t = time.perf_counter() - t0
    assert min(ms_calls) > 0.0, "drop-in entry point reported failure"
    e2e_value, e2e_t, _ = aggregate(ws, e2e_t, inter)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer sphere, G=M=a=1)",
        "config": {"workload": f"plain large system: N={n:,} Plummer, FP32 force, "
                               "FP64 KDK integrate, eps2=1e-4, dt=0.005",
                   "n_bodies": n, "integrator": "kdk64", "force_config": cfg_name,
                   "nsplit": nsplit,
                   "l2": "flushed between steps (256 MiB write outside the step events)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fp32_peak / 1e12,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu dram read+write, "
                                     "profiles/force_kernel_n1048576_dram.md)",
                     "algorithmic_bytes": 48 * n,  # read targets + sources, write forces
                     "peak_source": "measured on this GPU by nbgb_measure_peak "
                                    f"(FFMA {ffma / 1e12:.2f}, FFMA2 {ffma2 / 1e12:.2f} "
                                    "TFLOP/s; FMA = 2 FLOP)",
                     "kernel_ms": kernel_ms,
                     "mufu_peak_per_s": mufu,
                     "mufu_frac": (float(n) * float(n) / (kernel_ms * 1e-3)) / mufu},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": n * 16},
        "gpu_launches": 3 * args.steps,
        "clocks": clk,
        "wall_s": wall,
    }
    if args.force == "onesided" and not args.no_newton3:
        line["newton3"] = measure_newton3(args, n, p3, v3, pm_np, dev, ffma, ffma2, fp32_peak,
                                          flush)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        rate, el, info = cpu_rate(pm_np, args.cpu_seconds)
        line["cpu_baseline"] = dict(value=rate, unit=UNIT, **info)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_newton3(args, n, p3, v3, pm_np, dev, ffma, ffma2, fp32_peak, flush):
    """The same timed steps with the Newton's-third-law force variant (each
    pair evaluated once), reported beside the headline kernel."""
    import torch

    import nbody_gb300 as nb
    s = nb.System(n, nb.INTEGRATOR_KDK64, EPS2, DT, 1.0)
    s.set_state64(p3, v3, pm_np[:, 3].copy())
    s.set_force_algorithm("newton3")
    s.set_timing(True)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    for _ in range(args.warmup):
        s.step(1)
    s.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    fms = []
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[k][0].record(stream)
        s.step(1)
        ev[k][1].record(stream)
        fms.append(s.last_force_ms())
    torch.cuda.synchronize()
    s.synchronize()
    s.close()
    t = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    kms = float(np.mean(fms))
    return {"value": float(n) * n * args.steps / t / 1e9, "unit": UNIT,
            "ms_per_step": t * 1e3 / args.steps, "force_ms": kms,
            "roofline_20flop_frac": FLOP * float(n) * n / (kms * 1e-3) / fp32_peak,
            "executed_fp32_frac": 25 * (float(n) * n / 2) / (kms * 1e-3) / fp32_peak,
            "note": "each pair evaluated once and applied to both bodies (16 FP32 "
                    "operations = 25 FLOP per pair, FMA = 2, plus one rsqrt); the first "
                    "fraction uses the reference's 20 FLOP per interaction, the second the "
                    "FP32 work actually executed"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-newton3", action="store_true",
                    help="skip the extra Newton's-third-law measurement")
    ap.add_argument("--force", choices=["onesided", "newton3"], default="onesided",
                    help="force algorithm of the timed steps")
    ap.add_argument("--n", type=int, default=N_BODIES,
                    help="bodies (default 1,048,576; smaller only for profiling captures)")
    args = ap.parse_args()
    ws, rank, local = _dist()
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
