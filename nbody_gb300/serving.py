"""Serving: simulate(N, steps, seed) requests with continuous batching.

    python -m nbody_gb300.serving [--requests 20000] [--rates 10,inf] [--seed 5]
        [--n-lo 256] [--n-hi 65536] [--steps-lo 10] [--steps-hi 1000]
        [--dt 0.005] [--eps2 1e-4] [--budget-gb 120] [--slots 512]
        [--plain-sample N] [--work-budgets 2e10,1e10]

Requests arrive as a Poisson process (rate per second; inf = all at t = 0),
each with N log-uniform in [n_lo, n_hi], steps uniform in [steps_lo,
steps_hi] and a Plummer initial state from its own seed.

Batched server (continuous batching on nbgb_ensemble): a request that has
arrived is admitted at a tick boundary when a slot is free and its device
state fits the HBM state budget; large requests are admitted first come first
served while the active work per tick is below a work budget (about what
saturates the GPU), small requests join at once.  Admitted requests share
every tick (one persistent force launch for all of them); a request whose
steps are done is retired at the tick boundary, its final state is copied
back, and its slot and memory are freed for the next arrivals.  Latency =
completion time - arrival time.

Plain server (the comparison): the same stream served first-in first-out by
the single-system resident path (`System`), one request at a time.  Each
request's service time (state upload, steps, state download) is measured on
the GPU; completion times follow exactly from the FIFO rule
finish_k = max(arrival_k, finish_{k-1}) + service_k on the same arrival times.
With --plain-sample the service times of a seeded subsample are measured and
the rest are predicted from them per (N, steps) (stated in the result).
"""
from __future__ import annotations

import argparse
import json
import math
import time
from collections import deque

import numpy as np

# device bytes of one body's resident state in the ensemble arena (FP64 x,v;
# FP32 mass, posMass, acceleration, j-stream; split partials for up to 4)
BYTES_PER_BODY = 6 * 8 + 4 + 16 + 16 + 16 + 8 * 16


def make_requests(n_req: int, rate: float, seed: int, n_lo: int = 256, n_hi: int = 65536,
                  steps_lo: int = 10, steps_hi: int = 1000):
    rng = np.random.default_rng(seed)
    n = np.clip(np.rint(np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), n_req))), n_lo,
                n_hi).astype(int)
    steps = rng.integers(steps_lo, steps_hi + 1, n_req)
    gaps = rng.exponential(1.0, n_req)  # unit-rate gaps: same requests at every rate
    arrival = np.zeros(n_req) if math.isinf(rate) else np.cumsum(gaps / rate)
    seeds = rng.integers(1, 2 ** 62, n_req)
    return [{"id": k, "n": int(n[k]), "steps": int(steps[k]), "seed": int(seeds[k]),
             "arrival": float(arrival[k])} for k in range(n_req)]


def _initial_state(req):
    from . import ic_plummer
    p, v, pm, _ = ic_plummer(req["n"], req["seed"])
    return p, v, pm[:, 3].copy()


class BatchedServer:
    """Continuous batching over one ensemble arena."""

    def __init__(self, eps2: float = 1e-4, dt: float = 0.005, budget_bytes: float = 120e9,
                 max_slots: int = 512, max_bodies: int | None = None,
                 max_ticks_per_sync: int = 32, work_budget: float = 2e10,
                 small_work: float = 1e8):
        """work_budget: interactions per tick above which large requests wait
        (first come first served) instead of joining -- about what saturates
        the GPU, so joining would only slow everyone; requests whose own work
        per tick is below small_work always join (slots and memory allowing)."""
        from . import Ensemble
        self.dt = dt
        self.max_ticks_per_sync = max_ticks_per_sync
        self.work_budget = work_budget
        self.small_work = small_work
        self.budget = budget_bytes
        self.max_slots = max_slots
        if max_bodies is None:
            max_bodies = int(min(budget_bytes // BYTES_PER_BODY, 32 << 20))
        self.ens = Ensemble(max_bodies, max_slots, eps2)
        self.used_bytes = 0

    def close(self):
        self.ens.close()

    def run(self, requests, keep_states=(), time_limit: float | None = None):
        """Serve `requests` (dicts with n, steps, seed, arrival) in real time.
        Returns per-request records and, for ids in keep_states, final states.
        While a tick runs on the GPU the host prepares the initial states of
        requests that have arrived; admission happens at tick boundaries."""
        ens = self.ens
        pending = deque(sorted(requests, key=lambda r: r["arrival"]))
        ready = deque()  # arrived, initial state generated, not yet admitted
        running = {}
        records, states = {}, {}
        t0 = time.perf_counter()
        ticks = 0
        busy_s = 0.0

        def prepare(limit):
            now = time.perf_counter() - t0
            while pending and pending[0]["arrival"] <= now and len(ready) < limit:
                r = pending.popleft()
                ready.append((r, _initial_state(r)))

        remaining = {}  # slot -> ticks still to run (initial-force tick + steps)
        while pending or ready or running:
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                break
            prepare(self.max_slots - len(running) + 8)
            # admission: large requests first come first served while the
            # active work per tick is below the work budget; small ones always
            work = sum(float(x["n"]) ** 2 for x in running.values())
            k = 0
            while k < len(ready):
                r, (p, v, m) = ready[k]
                w = float(r["n"]) ** 2
                need = r["n"] * BYTES_PER_BODY
                if len(running) >= self.max_slots or self.used_bytes + need > self.budget:
                    break
                small = w <= self.small_work
                if not small and running and work + w > self.work_budget:
                    k += 1  # this one waits; later small ones may still join
                    continue
                slot = ens.add(p, v, m, self.dt, r["steps"])
                if slot is None:  # arena full: wait for retirements
                    break
                del ready[k]
                self.used_bytes += need
                work += w
                running[slot] = r
                remaining[slot] = r["steps"] + 1
                records[r["id"]] = {"n": r["n"], "steps": r["steps"], "arrival": r["arrival"],
                                    "admit": time.perf_counter() - t0}
            if not running:
                if pending and not ready:
                    wait = pending[0]["arrival"] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            # Run ticks until the next request finishes (known on the host),
            # bounded so arrivals are admitted within a few ticks.
            k = max(1, min(min(remaining.values()), self.max_ticks_per_sync))
            arrived = pending and pending[0]["arrival"] <= time.perf_counter() - t0
            if arrived and len(running) < self.max_slots:
                k = 1  # admit the newcomer at the next tick boundary
            tb = time.perf_counter()
            ens.tick(k)  # asynchronous
            prepare(self.max_slots - len(running) + 8)  # overlaps the ticks
            ens.synchronize()
            busy_s += time.perf_counter() - tb
            ticks += k
            for slot in remaining:
                remaining[slot] -= k
            for slot in ens.finished(self.max_slots):
                remaining.pop(slot, None)
                r = running.pop(slot)
                st = ens.get_state(slot)  # the result goes back to the client
                if r["id"] in keep_states:
                    states[r["id"]] = st
                ens.remove(slot)
                self.used_bytes -= r["n"] * BYTES_PER_BODY
                rec = records[r["id"]]
                rec["finish"] = time.perf_counter() - t0
                rec["latency"] = rec["finish"] - rec["arrival"]
        wall = time.perf_counter() - t0
        return records, states, {"wall_s": wall, "ticks": ticks, "host_and_gpu_tick_s": busy_s}


def plain_service_time(req, eps2: float, dt: float) -> float:
    import torch

    from . import INTEGRATOR_KDK64, System
    p, v, m = _initial_state(req)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = System(req["n"], INTEGRATOR_KDK64, eps2, dt, 1.0)
    s.set_state64(p, v, m)
    s.step(req["steps"])
    s.get_state64()
    s.close()
    return time.perf_counter() - t0


def fifo_finish_times(arrivals, service):
    finish, t = [], 0.0
    for a, s in zip(arrivals, service):
        t = max(t, a) + s
        finish.append(t)
    return finish


def _pct(x, q):
    return float(np.percentile(np.asarray(x), q)) if len(x) else None


def _batched_run(reqs, eps2, dt, budget_gb, slots, work_budget=2e10):
    srv = BatchedServer(eps2, dt, budget_gb * 1e9, slots, work_budget=work_budget)
    recs, _, info = srv.run(reqs)
    srv.close()
    lat = [r["latency"] for r in recs.values() if "latency" in r]
    inter = sum(float(r["n"]) ** 2 * (r["steps"] + 1) for r in recs.values() if "latency" in r)
    span = max(r["finish"] for r in recs.values() if "finish" in r) - min(
        r["arrival"] for r in reqs)
    return {"completed": len(lat), "wall_s": info["wall_s"], "ticks": info["ticks"],
            "tick_loop_s": info["host_and_gpu_tick_s"], "systems_per_s": len(lat) / span,
            "interactions_per_s": inter / span, "latency_p50_s": _pct(lat, 50),
            "latency_p99_s": _pct(lat, 99),
            "latency_mean_s": float(np.mean(lat)) if lat else None,
            "work_budget": work_budget}


def serve_study(n_req: int = 20000, rates=(10.0,), seed: int = 5, n_lo: int = 256,
                n_hi: int = 65536, steps_lo: int = 10, steps_hi: int = 1000, dt: float = 0.005,
                eps2: float = 1e-4, budget_gb: float = 120.0, slots: int = 512,
                plain_sample: int | None = None, work_budgets=(2e10,)) -> dict:
    """Both servers on the same stream at each arrival rate.  The plain
    server's per-request service times are measured once (they do not depend
    on the arrival times) and replayed through the FIFO rule at every rate.
    The batched server runs once per work budget (interactions per tick
    above which large requests wait); the first budget is the headline."""
    base = make_requests(n_req, 1.0, seed, n_lo, n_hi, steps_lo, steps_hi)
    rng = np.random.default_rng(seed + 17)
    if plain_sample is None or plain_sample >= n_req:
        idx = list(range(n_req))
    else:
        idx = sorted(rng.choice(n_req, plain_sample, replace=False).tolist())
    measured = {k: plain_service_time(base[k], eps2, dt) for k in idx}
    if len(measured) == n_req:
        service = [measured[k] for k in range(n_req)]
    else:
        # fit service = c0 + c1 * steps + c2 * steps * N^2 on the sample
        A = np.array([[1.0, base[k]["steps"], base[k]["steps"] * base[k]["n"] ** 2]
                      for k in idx])
        y = np.array([measured[k] for k in idx])
        coef, *_ = np.linalg.lstsq(A, y, rcond=None)
        service = [measured.get(k, float(coef @ [1.0, r["steps"], r["steps"] * r["n"] ** 2]))
                   for k, r in enumerate(base)]
    out = {"study": "serving", "requests": n_req, "seed": seed, "n_range": [n_lo, n_hi],
           "steps_range": [steps_lo, steps_hi], "dt": dt, "softeningSquared": eps2,
           "budget_gb": budget_gb, "slots": slots,
           "plain_service_total_s": float(sum(service)),
           "plain_measured_requests": len(measured),
           "plain_service_predicted": len(measured) != n_req, "by_rate": []}
    for rate in rates:
        reqs = make_requests(n_req, rate, seed, n_lo, n_hi, steps_lo, steps_hi)
        runs = [_batched_run(reqs, eps2, dt, budget_gb, slots, wb) for wb in work_budgets]
        b = runs[0]
        arrivals = [r["arrival"] for r in reqs]
        pfin = fifo_finish_times(arrivals, service)
        plat = [f - a for f, a in zip(pfin, arrivals)]
        pspan = pfin[-1] - arrivals[0]
        p = {"systems_per_s": n_req / pspan, "latency_p50_s": _pct(plat, 50),
             "latency_p99_s": _pct(plat, 99), "latency_mean_s": float(np.mean(plat))}
        row = {"rate_per_s": rate, "batched": b, "plain": p,
               "speedup_systems_per_s": b["systems_per_s"] / p["systems_per_s"]}
        if len(runs) > 1:
            row["batched_other_work_budgets"] = runs[1:]
        out["by_rate"].append(row)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=20000)
    ap.add_argument("--rates", default="10",
                    help="comma-separated arrival rates per second (inf = all at t = 0)")
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--n-lo", type=int, default=256)
    ap.add_argument("--n-hi", type=int, default=65536)
    ap.add_argument("--steps-lo", type=int, default=10)
    ap.add_argument("--steps-hi", type=int, default=1000)
    ap.add_argument("--dt", type=float, default=0.005)
    ap.add_argument("--eps2", type=float, default=1e-4)
    ap.add_argument("--budget-gb", type=float, default=120.0)
    ap.add_argument("--slots", type=int, default=512)
    ap.add_argument("--plain-sample", type=int, default=None)
    ap.add_argument("--work-budgets", default="2e10",
                    help="comma-separated interactions per tick above which large requests "
                         "wait; the batched server runs once per value, the first is the "
                         "headline")
    a = ap.parse_args(argv)
    rates = [float(x) for x in a.rates.split(",")]
    budgets = [float(x) for x in a.work_budgets.split(",")]
    r = serve_study(a.requests, rates, a.seed, a.n_lo, a.n_hi, a.steps_lo, a.steps_hi, a.dt,
                    a.eps2, a.budget_gb, a.slots, a.plain_sample, budgets)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
