"""Autotuner for the ensemble force pass: per N bucket, the kernel variant
(targets per thread and unroll), the tile size and the j-split.

    python -m nbody_gb300.autotune [--buckets 6-16] [--out PATH]

For each bucket b (N in [2^b, 2^(b+1))) it builds an ensemble of identical
systems of N = 2^(b+0.5) bodies (uniform ball, seeded), enough of them for a
tick of ~2e9 interactions and several waves of work items, and times a few
ticks of every candidate plan with
CUDA-synchronised host timing; the fastest plan per bucket is written to a
JSON table.  Ensemble(tuning="auto") applies nbody_gb300/tuning/ensemble.json
when it exists.  Plans only change speed, never results beyond rounding, and a
system's plan still depends only on its own N.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

TUNING_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")
DEFAULT_PATH = os.path.join(TUNING_DIR, "ensemble.json")

VARIANTS = {0: (1, 8), 1: (2, 4), 2: (1, 4), 3: (2, 8)}  # targets/thread, unroll


def candidates(n: int):
    out = []
    for variant in VARIANTS:
        for jt in (128, 256, 512, 1024):
            if jt > max(128, 2 * n):
                continue  # tiles far larger than the system are mostly padding
            splits = (1, 2, 4) if n >= 4096 else (1,)
            for nsplit in splits:
                out.append((variant, jt, nsplit))
    return out


def time_plan(n: int, plan, n_systems: int, ticks: int, seed: int = 7) -> float:
    import nbody_gb300 as nb
    e = nb.Ensemble(n * n_systems, n_systems, 1e-4, tuning=None)
    b = nb.bucket_of(n)
    e.set_bucket_plan(b, *plan)
    for k in range(n_systems):
        pm, _ = nb.ic_uniform_ball(n, seed + k, 1.0, 0.5, 1.5)
        p = pm[:, :3].astype(np.float64)
        slot = e.add(p, np.zeros_like(p), pm[:, 3].copy(), 1e-3, ticks + 1)
        if slot is None:
            raise RuntimeError(f"ensemble admission failed for plan {plan} at N={n}")
    e.tick(1)
    e.synchronize()
    t0 = time.perf_counter()
    e.tick(ticks)
    e.synchronize()
    dt = (time.perf_counter() - t0) / ticks
    e.close()
    return dt


def tune(buckets=range(6, 17), ticks: int = 4, verbose: bool = True) -> dict:
    import torch
    table = {"device": torch.cuda.get_device_name(0), "buckets": {}}
    for b in buckets:
        n = int(round(2 ** (b + 0.5)))
        # enough systems for ~2e9 interactions per tick and for ~4 waves of
        # 512-body items over the GPU's CTA slots, as in a real mix
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        n_systems = int(max(2, min(1024, max(2e9 / (n * n), 4 * sms * 2 * 512 / n))))
        best = None
        for plan in candidates(n):
            t = time_plan(n, plan, n_systems, ticks)
            rate = n_systems * n * n / t
            if verbose:
                print(f"bucket {b:2d} N={n:6d} x{n_systems:4d} plan {plan}: "
                      f"{t * 1e3:8.3f} ms/tick {rate / 1e9:8.1f} G/s", flush=True)
            if best is None or t < best[0]:
                best = (t, plan, rate)
        table["buckets"][str(b)] = {"variant": best[1][0], "jt": best[1][1],
                                    "nsplit": best[1][2], "n": n, "systems": n_systems,
                                    "ms_per_tick": best[0] * 1e3,
                                    "interactions_per_s": best[2]}
    return table


def load(path: str = DEFAULT_PATH):
    if path and os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return None


def apply(ens, table) -> None:
    if not table:
        return
    for b, plan in table.get("buckets", {}).items():
        ens.set_bucket_plan(int(b), plan["variant"], plan["jt"], plan["nsplit"])


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--buckets", default="6-16")
    ap.add_argument("--ticks", type=int, default=4)
    ap.add_argument("--out", default=DEFAULT_PATH)
    a = ap.parse_args(argv)
    lo, hi = (int(x) for x in a.buckets.split("-"))
    table = tune(range(lo, hi + 1), a.ticks)
    os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps(table))


if __name__ == "__main__":
    main()
