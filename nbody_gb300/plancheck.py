"""Check the single-system force planner on this GPU.

    python -m nbody_gb300.plancheck [--sizes 1000,4096,...] [--calls 5]

For each N (a seeded Plummer sphere) it times the planner's own plan for
nbgb_force and a grid of forced plans (configuration x slice count: every
i-block split s ways, and from N = 131,072 also whole i-blocks for the whole
rounds of CTA slots plus the leftover i-blocks split s ways, nsplit = -s),
each as a CUDA graph of `calls` back-to-back calls (the pack and force
kernels, no host work in the timed region), and prints one JSON line per N:
the planner's plan and time, the fastest three grid plans and the planner's
time over the fastest.  Plans change speed only; results differ at most by
rounding.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

DEFAULT_SIZES = (1000, 2048, 3000, 4096, 6000, 8192, 10007, 12000, 16384, 20000, 32768, 50000,
                 65536, 100000, 131072, 155677, 200000, 262144, 524288, 1048576)
GRID_CONFIGS = ("w8_k2_jt1024_s3_log4", "w4_k2_jt256_s4_log4", "w8_k2_jt256_s4_log4",
                "w8_k2_jt2048_s2_log4", "w6_k3_jt1024_s2_log4")
GRID_SPLITS = (1, 4, 8, 16, 32)
TAIL_SPLITS = (-8, -16, -32)  # leftover i-blocks only, from N = 131,072


def graph_time_us(pm, out, config: int, nsplit: int, calls: int, reps: int = 3) -> float:
    """Median microseconds per call of nbgb_force over `reps` replays of a
    graph of `calls` calls."""
    import torch

    from . import Workspace, force
    ws = Workspace()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        force(pm, 1e-4, out=out, config=config, nsplit=nsplit, workspace=ws)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=side):
        for _ in range(calls):
            force(pm, 1e-4, out=out, config=config, nsplit=nsplit, workspace=ws)
    g.replay()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) / calls)
    return float(np.median(ts)) * 1e3


def check(n: int, calls: int = 5) -> dict:
    import torch

    from . import force_config_names, force_plan, ic_plummer, last_status
    names = force_config_names()
    _, _, pm_np, _ = ic_plummer(n, 20260)
    pm = torch.from_numpy(pm_np).cuda()
    out = torch.empty_like(pm)
    cfg, nsplit, wsb = force_plan(n)
    t_plan = graph_time_us(pm, out, -1, -1, calls)
    large = n > 262144  # few grid points: these sizes take 0.1-0.4 s a call
    tails = TAIL_SPLITS if n >= 131072 else ()
    grid = []
    for ci, name in enumerate(GRID_CONFIGS[:1] if large else GRID_CONFIGS):
        c = names.index(name)
        for s in ((8, 16) if large else GRID_SPLITS) + (tails if ci == 0 else ()):
            _, s_eff, _ = force_plan(n, c, s)
            if s_eff != abs(s):
                continue  # fewer j-tiles than slices
            grid.append((graph_time_us(pm, out, c, s, 2 if large else calls), name, s))
    grid.sort()
    if last_status() != 0:
        raise RuntimeError(f"device status {last_status()} at N = {n}")
    return {"n": n, "plan": {"config": names[cfg], "nsplit": nsplit, "workspace_bytes": wsb,
                             "us": round(t_plan, 2)},
            "grid_best": [{"config": nm, "nsplit": s, "us": round(u, 2)} for u, nm, s in grid[:3]],
            "plan_over_best": round(t_plan / grid[0][0], 4) if grid else None}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default=",".join(str(n) for n in DEFAULT_SIZES))
    ap.add_argument("--calls", type=int, default=5)
    a = ap.parse_args(argv)
    for n in (int(x) for x in a.sizes.split(",")):
        print(json.dumps(check(n, a.calls)), flush=True)


if __name__ == "__main__":
    main()
