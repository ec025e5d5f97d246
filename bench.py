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
            stream, L2 flushed (a 256 MiB read, which leaves no dirty lines
            behind) between steps outside the events
  e2e       the reference-facing drop-in ComputeGravitation_GPU_GB300 with
            HOST buffers: per step pinned H2D of posMass, the call, D2H of the
            forces, all inside a host-clock timed region
  roofline  the force kernel: 20 N^2 FLOP / its CUDA-event launch time, over
            the FP32 pipe peak measured by the library's FMA microbenchmark
            on this GPU (max of scalar and f32x2), plus the MUFU ceiling;
            `integrate` holds the same for the HBM-bound integrate kernels:
            the FP64 kick+drift and half kick of the resident loop and the
            reference-mode step (algorithmic bytes / CUDA-event time over the
            measured copy bandwidth)
  cpu_baseline  the oracle's restatement of the reference's CPU_SOA loop
            (OpenMP, all host threads) on a bounded sample of target bodies
            against all N sources
  accuracy  the drop-in's forces of the e2e leg on a seeded 1,024-body
            sample, per body against the FP64 all-pairs sum and against the
            oracle's CPU_AOS restatements (IEEE and the reference's flags),
            computed outside every timed region
  reference_mode  milliseconds per resident reference-mode step on small
            plain systems (N = 1,024, 4,096, 16,384): one launch per step
            (the integrate in the force kernel's epilogue) against force
            then integrate, both replaying CUDA graphs of 8 steps

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
                      f"CPU_SOA (src/nbody_CPU_SOA.cpp:53-105) built with {O.fast_flags()} "
                      "(the reference's flags, meson.build:33-58)"}
    return rate, el, info


TRAFFIC_TABLE = os.path.join(ROOT, "nbody_gb300", "tuning", "force_dram_traffic.json")
# measured copy bandwidth of this GPU type when MEASURED_PEAKS.json is absent
HBM_FALLBACK_GBS = 6800.0


def profiled_traffic(config_name: str, n: int, nsplit: int):
    """DRAM bytes per force launch measured by ncu for this kernel
    configuration, N and j-split (nbody_gb300/tuning/force_dram_traffic.json),
    else None."""
    try:
        table = json.load(open(TRAFFIC_TABLE))
    except (OSError, ValueError):
        return None
    for e in table.get("entries", []):
        if e["config"] == config_name and e["n"] == n and e["nsplit"] == nsplit:
            return int(e["bytes_per_launch"])
    return None


def hbm_peak():
    """(GB/s, source): the measured copy bandwidth, else the fallback."""
    try:
        v = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
        return v, "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except (OSError, ValueError, KeyError, TypeError):
        return HBM_FALLBACK_GBS, "fallback (6.8 TB/s, one earlier GB300 measurement)"


def run_reference_arm(args, ws, rank):
    """The reference's CPU path alone: the oracle's restatement of CPU_SOA
    built with the reference's flags, on inputs from the oracle's restatement
    of the Plummer generator (byte-identical to the library's, tested), so
    this arm loads no GB300 code."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build(ref=False)
    _, _, pm = O.ieee().ic_plummer(N_BODIES, SEED)
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
                                   "of the reference's CPU_SOA (src/nbody_CPU_SOA.cpp:53-105) "
                                   f"built with {O.fast_flags()} (the reference's flags, "
                                   "meson.build:33-58; its own CPU objects are built only "
                                   "where its sources are present, and tests check the "
                                   "restatement against them)"},
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
    flush = L2Flush(dev)

    for _ in range(args.warmup):
        sysm.step(1)
    sysm.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    force_ms, kd_ms, hk_ms = [], [], []
    clocks = Clocks(int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[0])
                    if os.environ.get("CUDA_VISIBLE_DEVICES", "").isdigit() else local)
    _barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush()  # evict L2 between steps (outside the events)
            ev[k][0].record(stream)
        sysm.step(1)
        ev[k][1].record(stream)
        force_ms.append(sysm.last_force_ms())
        kd_ms.append(sysm.last_integrate_ms()[0])
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
    # the closing half kick runs only when velocities are read (or merges
    # into the next step's kick): time it on its own, outside the steps
    for _ in range(3):
        sysm.step(1)
        with torch.cuda.stream(stream):
            flush()
        sysm.sync_velocities()
        hk_ms.append(sysm.last_integrate_ms()[1])
    cfg, nsplit = sysm.plan()
    cfg_name = nb.force_config_names()[cfg] if args.force == 'onesided' else 'newton3'
    traffic = profiled_traffic(cfg_name, n, nsplit)
    sysm.close()
    integrate = integrate_roofline(n, kd_ms, hk_ms,
                                   reference_step_ms(n, dev, torch.cuda.current_stream(), flush))

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
                   "l2": "flushed between steps (256 MiB read outside the step events)",
                   "parallelism": f"replicas x{ws}"},
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fp32_peak / 1e12,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                     "traffic_unit": "bytes per launch (ncu dram read+write, "
                                     "nbody_gb300/tuning/force_dram_traffic.json)",
                     "algorithmic_bytes": 48 * n,  # read targets + sources, write forces
                     "peak_source": "measured on this GPU by nbgb_measure_peak "
                                    f"(FFMA {ffma / 1e12:.2f}, FFMA2 {ffma2 / 1e12:.2f} "
                                    "TFLOP/s; FMA = 2 FLOP)",
                     "kernel_ms": kernel_ms,
                     "mufu_peak_per_s": mufu,
                     "mufu_frac": (float(n) * float(n) / (kernel_ms * 1e-3)) / mufu,
                     "integrate": integrate},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": n * 16},
        "gpu_launches": 2 * args.steps,  # per step: kick+drift, force
        "clocks": clk,
        "wall_s": wall,
    }
    if args.force == "onesided" and not args.no_newton3:
        line["newton3"] = measure_newton3(args, n, p3, v3, pm_np, dev, ffma, ffma2, fp32_peak,
                                          flush)
    try:
        line["reference_mode"] = [reference_mode_steps(dev, m) for m in (1024, 4096, 16384)]
    except Exception as e:  # a side measurement: keep the line
        line["reference_mode"] = {"error": f"{type(e).__name__}: {e}"[:300]}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        rate, el, info = cpu_rate(pm_np, args.cpu_seconds)
        line["cpu_baseline"] = dict(value=rate, unit=UNIT, **info)
        line["accuracy"] = force_accuracy(pm_np, f_h.numpy())
    if rank == 0:
        print(json.dumps(line), flush=True)


class L2Flush:
    """Evicts L2 (129 MB on GB300) by reading a 256 MiB buffer: a read leaves
    clean lines, so the next kernel pays no write-back of the flush itself."""

    def __init__(self, dev):
        import torch
        self.buf = torch.ones(64 << 20, dtype=torch.int32, device=dev)

    def __call__(self):
        self.buf.amax()


# bytes each FP64 integrate kernel moves per body (algorithmic: every array
# read and written once)
KICK_DRIFT_BYTES = 148  # read x, v (48), a (16), m (4); write x, v (48), posMass, j-stream (32)
HALF_KICK_BYTES = 64    # read v (24), a (16); write v (24)
REFERENCE_STEP_BYTES = 80  # read posMass, velInvMass, force; write posMass, velInvMass


def reference_step_ms(n, dev, stream, flush, reps=5):
    """CUDA-event times of the reference-mode integrate (integrateOne on the
    GPU, nbgb_integrate_reference) on N bodies of device arrays, each launch
    right after the L2 flush."""
    import torch

    import nbody_gb300 as nb
    g = torch.Generator(device="cpu").manual_seed(3)
    pm = torch.rand((n, 4), generator=g).to(dev)
    vm = torch.rand((n, 4), generator=g).to(dev)
    f = torch.rand((n, 4), generator=g).to(dev)
    out = []
    for _ in range(reps + 1):
        with torch.cuda.stream(stream):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            nb.integrate_reference(pm, vm, f, 1e-6, 0.95, stream=stream.cuda_stream)
            e1.record(stream)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return out[1:]


def reference_mode_steps(dev, n=16384, steps=400):  # steps: a multiple of 8
    """Milliseconds per reference-mode step on the plain case at N bodies
    (uniform ball, eps2 = 1e-4, dt = 0.01, damping 0.95, contracted drift):
    the System's resident loop, one launch per step (the integrate runs in
    the force kernel's epilogue; graph-launched), against the two-launch form
    (standalone force kernel, then integrateOne), both replaying CUDA graphs
    of 8 steps.  L2-resident state: this is the launch and tail cost the
    fusion removes, not an HBM figure."""
    import torch

    import nbody_gb300 as nb
    pm, vm = nb.ic_uniform_ball(n, 16384)
    s = nb.System(n, nb.INTEGRATOR_REFERENCE_FUSED, 1e-4, 0.01, 0.95)
    s.set_state(pm, vm)
    st = torch.cuda.ExternalStream(s.stream, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.step(8)
    s.synchronize()
    e0.record(st)
    s.step(steps)
    e1.record(st)
    s.synchronize()
    fused_ms = e0.elapsed_time(e1) / steps
    s.close()
    tp = torch.from_numpy(pm).to(dev)
    tv = torch.from_numpy(vm).to(dev)
    f = torch.empty_like(tp)
    ws = nb.Workspace()
    side = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(side):
        for _ in range(3):  # plans the workspace outside the capture
            nb.force(tp, 1e-4, out=f, workspace=ws)
            nb.integrate_reference(tp, tv, f, 0.01, 0.95, fused_drift=True)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        for _ in range(8):
            nb.force(tp, 1e-4, out=f, workspace=ws)
            nb.integrate_reference(tp, tv, f, 0.01, 0.95, fused_drift=True)
    g.replay()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps // 8):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    two_ms = e0.elapsed_time(e1) / steps
    return {"n_bodies": n, "steps": steps, "ms_per_step_one_launch": fused_ms,
            "ms_per_step_two_launches": two_ms, "speedup": two_ms / fused_ms,
            "state": f"L2-resident (4 arrays x {n * 16 // 1024} KiB)"}


def integrate_roofline(n, kd_ms, hk_ms, ref_ms=()):
    """HBM roofline of the integrate kernels from CUDA-event times, each
    launched right after the L2 flush (cold state): the FP64 kick+drift of
    every timed step, the closing half kick, which runs only when the
    velocities are read (timed three times after the steps), and the
    reference-mode step (integrateOne) on the same N."""
    peak, src = hbm_peak()
    out = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": src}
    for name, per_body, ms in (("kick_drift", KICK_DRIFT_BYTES, kd_ms),
                               ("half_kick", HALF_KICK_BYTES, hk_ms),
                               ("reference_step", REFERENCE_STEP_BYTES, ref_ms)):
        t = float(np.median(ms)) if ms else 0.0
        gbs = per_body * float(n) / (t * 1e-3) / 1e9 if t > 0 else None
        out[name] = {"bytes_per_body": per_body, "bytes": per_body * n, "ms": t,
                     "achieved": gbs, "frac": gbs / peak if gbs else None}
    return out


def force_accuracy(pm: np.ndarray, force: np.ndarray, k: int = 1024, seed: int = 7):
    """Per-body |F - T| / |T| of `force` on a seeded sample of k bodies: T the
    FP64 all-pairs sum of the same FP32 inputs; the reference's compiled
    CPU_AOS (src/nbody_CPU_AOS.cpp:51-98) from its fixture; and the CPU_AOS
    restatement built on this host IEEE (sequential sum: at N = 2^20 itself
    ~1e-4 from FP64) and with the reference's flags (given also net of its
    own distance from FP64: on aarch64 its reciprocal square root is
    low-precision)."""
    from oracle import oracle as O
    n = pm.shape[0]
    idx = np.random.default_rng(seed).choice(n, min(k, n), replace=False)
    f = np.asarray(force, np.float64)[idx, :3]
    t64 = O.ieee().forces_f64(pm, float(np.float32(EPS2)), idx)

    def stats(ref):
        d = np.linalg.norm(f - ref, axis=1) / np.linalg.norm(ref, axis=1)
        return {"max": float(d.max()), "rms": float(np.sqrt(np.mean(d * d)))}

    ieee = O.ieee().forces_aos_idx(pm, EPS2, idx)[:, :3].astype(np.float64)
    fast = O.fast().forces_aos_idx(pm, EPS2, idx)[:, :3].astype(np.float64)
    net = (np.linalg.norm(f - fast, axis=1) - np.linalg.norm(fast - t64, axis=1)) / \
        np.linalg.norm(fast, axis=1)
    out = {"sample": f"{idx.size} seeded bodies of the N={n:,} input, forces of the "
                     "drop-in call (e2e leg)",
           "vs_fp64": stats(t64)}
    # the reference's own compiled CPU_AOS on this input, when its forces for
    # this sample are on file (made where the reference builds)
    fx = os.path.join(ROOT, "tests", "golden", "c2_plummer1m_sample.npz")
    if os.path.exists(fx):
        import hashlib
        g = np.load(fx)
        if (int(g["n"]) == n and np.array_equal(g["idx"], idx) and
                hashlib.sha256(np.ascontiguousarray(pm).tobytes()).hexdigest() ==
                g["posMass_sha256"].item().decode()):
            out["vs_reference_compiled_cpu_aos"] = dict(
                stats(g["force_aos"][:, :3].astype(np.float64)),
                source="tests/golden/c2_plummer1m_sample.npz (the reference's "
                       "ComputeGravitation_AOS built with its flags on x86-64)")
    return dict(out, **{
            "vs_cpu_aos_ieee": stats(ieee),
            "vs_cpu_aos_reference_flags": dict(stats(fast),
                                               net_of_own_fp64_distance_max=float(
                                                   max(0.0, net.max())),
                                               flags=O.fast_flags()),
            "gates": {"vs_reference_max": 1e-5, "vs_fp64_max": 5e-6}})


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
            flush()
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
