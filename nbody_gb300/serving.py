"""Serving: simulate(N, steps, seed) requests with continuous batching.

    python -m nbody_gb300.serving [--requests 20000] [--rates 10,inf] [--seed 5]
        [--n-lo 256] [--n-hi 65536] [--steps-lo 10] [--steps-hi 1000]
        [--dt 0.005] [--eps2 1e-4] [--budget-gb 120] [--slots 512]
        [--plain-sample N] [--work-budgets 2e10,1e10] [--sub-work 0]
        [--express-n 8192] [--express-ctas 32] [--newton3-min 16384] [--records PATH]

Requests arrive as a Poisson process (rate per second; inf = all at t = 0),
each with N log-uniform in [n_lo, n_hi], steps uniform in [steps_lo,
steps_hi] and a Plummer initial state from its own seed.

Batched server (continuous batching on nbgb_ensemble): a request that has
arrived is admitted at a tick boundary when a slot is free and its device
state fits the HBM state budget; large requests are admitted first come first
served while the active work per tick is below a work budget (about what
saturates the GPU), small requests join at once.  Admitted requests share
every tick (one persistent force launch per step level for all of them);
small requests take up to 8 steps per tick (ensemble sub-cycling), so
they are not held to the pace of the large ones; a request whose
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
BYTES_PER_BODY = 6 * 8 + 4 + 16 + 16 + 16 + 8 * 16 + 3 * 8  # + FP64 Newton-3 sums


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


class _Lane:
    """One ensemble arena with its own stream, admission state and loop."""

    def __init__(self, ens, budget_bytes, max_slots, dt, max_ticks_per_sync, work_budget,
                 small_work, sub_work):
        self.ens = ens
        self.budget = budget_bytes
        self.max_slots = max_slots
        self.dt = dt
        self.max_ticks_per_sync = max_ticks_per_sync
        self.work_budget = work_budget
        self.small_work = small_work
        self.sub_work = sub_work
        self.used_bytes = 0

    def _sub(self, n: int) -> int:
        return int(max(1, min(8, self.sub_work // (float(n) ** 2))))

    def serve(self, requests, t0, keep_states=(), time_limit=None):
        """Serve `requests` (arrival times relative to t0) in real time.
        While a tick runs on the GPU the host prepares the initial states of
        requests that have arrived; admission happens at tick boundaries."""
        ens = self.ens
        pending = deque(sorted(requests, key=lambda r: r["arrival"]))
        ready = deque()  # arrived, initial state generated, not yet admitted
        running = {}
        records, states = {}, {}
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
            # large requests' work per step is below the work budget; small
            # ones always join and do not count against it
            work = sum(float(x["n"]) ** 2 for x in running.values()
                       if float(x["n"]) ** 2 > self.small_work)
            k = 0
            large_blocked = False  # strict FCFS among large requests
            while k < len(ready):
                r, (p, v, m) = ready[k]
                w = float(r["n"]) ** 2
                need = r["n"] * BYTES_PER_BODY
                if len(running) >= self.max_slots or self.used_bytes + need > self.budget:
                    break
                small = w <= self.small_work
                if not small and (large_blocked or (work > 0 and work + w > self.work_budget)):
                    # this one waits, and so does every large request behind it
                    # (no overtaking, so the largest requests cannot starve);
                    # later small ones may still join
                    large_blocked = True
                    k += 1
                    continue
                slot = ens.add(p, v, m, self.dt, r["steps"])
                if slot is None:  # arena full: wait for retirements
                    break
                sub = self._sub(r["n"])
                if sub > 1:
                    ens.set_substeps(slot, sub)
                del ready[k]
                self.used_bytes += need
                if not small:
                    work += w
                running[slot] = r
                remaining[slot] = 1 + -(-r["steps"] // sub)  # initial forces + ticks
                records[r["id"]] = {"n": r["n"], "steps": r["steps"], "arrival": r["arrival"],
                                    "admit": time.perf_counter() - t0}
            if not running:
                if pending and not ready:
                    wait = pending[0]["arrival"] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.005))
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
        return records, states, {"ticks": ticks, "host_and_gpu_tick_s": busy_s}


class BatchedServer:
    """Continuous batching: a main lane (one ensemble arena) and, for small
    requests, an express lane (a second ensemble on its own stream whose
    persistent force launch holds a few CTA slots that the main lane leaves
    free), so small requests run at their own tick pace beside the large
    ones instead of in lockstep with them."""

    def __init__(self, eps2: float = 1e-4, dt: float = 0.005, budget_bytes: float = 120e9,
                 max_slots: int = 512, max_bodies: int | None = None,
                 max_ticks_per_sync: int = 32, work_budget: float = 2e10,
                 small_work: float = 1e8, sub_work: float = 0.0, express_n: int = 8192,
                 express_ctas: int = 32, express_slots: int = 256, newton3_min: int = 16384,
                 ensemble_factory=None):
        """work_budget: interactions per step of the large requests running
        above which further large requests wait (first come first served)
        instead of joining -- about what saturates the GPU, so joining would
        only slow everyone; small requests (N^2 <= small_work) always join
        (slots and memory allowing) and do not count against it.
        sub_work: a request takes sub = min(8, sub_work // N^2) (at least 1)
        steps per tick (0: one step per tick).
        express_n: requests with N <= express_n go to the express lane
        (express_ctas CTA slots, express_slots systems); 0 = one lane.
        newton3_min: main-lane requests with N >= newton3_min are evaluated
        with the Newton's-third-law kernel (0: none).
        ensemble_factory(max_bodies, max_systems, eps2): the arena type
        (default nbody_gb300.Ensemble; tests pass a host-side stand-in)."""
        if ensemble_factory is None:
            from . import Ensemble as ensemble_factory
        self.dt = dt
        self.budget = budget_bytes
        self.max_slots = max_slots
        self.express = None
        self.express_n = express_n
        ex_budget = 0.0
        if express_n > 0:
            ex_budget = min(budget_bytes / 4, express_slots * express_n * BYTES_PER_BODY)
            ex = ensemble_factory(express_slots * express_n, express_slots, eps2)
            ex.set_grid(express_ctas)
            ex.set_priority(True)  # ahead of the main lane's pending CTAs
            self.express = _Lane(ex, ex_budget, express_slots, dt, max_ticks_per_sync,
                                 work_budget, small_work, sub_work)
        main_budget = budget_bytes - ex_budget
        if max_bodies is None:
            max_bodies = int(min(main_budget // BYTES_PER_BODY, 32 << 20))
        ens = ensemble_factory(max_bodies, max_slots, eps2)
        if self.express is not None:
            ens.set_grid(ens.max_grid() - express_ctas)
        if newton3_min > 0:
            ens.set_newton3_min(newton3_min)
        self.main = _Lane(ens, main_budget, max_slots, dt, max_ticks_per_sync, work_budget,
                          small_work, sub_work)
        self.ens = ens  # the main lane's ensemble

    @property
    def used_bytes(self):
        return self.main.used_bytes + (self.express.used_bytes if self.express else 0)

    def close(self):
        self.main.ens.close()
        if self.express is not None:
            self.express.ens.close()

    def run(self, requests, keep_states=(), time_limit: float | None = None):
        """Serve `requests` (dicts with n, steps, seed, arrival) in real time.
        Returns per-request records and, for ids in keep_states, final states.
        The lanes run in two host threads (the library's calls release the
        interpreter lock); latency = completion time - arrival time."""
        import threading
        if self.express is not None:
            small = [r for r in requests if r["n"] <= self.express_n]
            large = [r for r in requests if r["n"] > self.express_n]
        else:
            small, large = [], list(requests)
        t0 = time.perf_counter()
        out = {}
        errors = []

        def express_lane():
            try:
                out["express"] = self.express.serve(small, t0, keep_states, time_limit)
            except BaseException as exc:  # re-raised in the caller's thread
                errors.append(exc)

        th = None
        if small:
            th = threading.Thread(target=express_lane)
            th.start()
        out["main"] = self.main.serve(large, t0, keep_states, time_limit)
        if th is not None:
            th.join()
        if errors:
            raise errors[0]
        records, states, info = {}, {}, {"wall_s": time.perf_counter() - t0, "ticks": 0,
                                         "host_and_gpu_tick_s": 0.0, "lanes": {}}
        for name, (rec, st, inf) in out.items():
            records.update(rec)
            states.update(st)
            info["ticks"] += inf["ticks"]
            info["host_and_gpu_tick_s"] += inf["host_and_gpu_tick_s"]
            info["lanes"][name] = dict(inf, requests=len(rec))
        return records, states, info


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


def best_interaction_rate(n: int = 1 << 20, eps2: float = 1e-4, reps: int = 3) -> dict:
    """The fastest force evaluation this GPU runs, in interactions/s: the
    one-sided and the Newton's-third-law kernels on a full N = 2^20 Plummer
    sphere (large enough that every SM is busy), best of `reps` each.  No
    request of any size can be served faster than this rate."""
    import torch

    from . import force, force_newton3, ic_plummer
    _, _, pm_np, _ = ic_plummer(n, 1)
    pm = torch.from_numpy(pm_np).cuda()
    out = {}
    for name, fn in (("onesided", force), ("newton3", force_newton3)):
        fn(pm, eps2)
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(pm, eps2)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        out[name] = float(n) * n / best
    out["best"] = max(out["onesided"], out["newton3"])
    return out


def throughput_bound(reqs, service, best_rate: float) -> dict:
    """Upper bound of the batched server's systems/s over the plain FIFO
    server's when both are saturated: the plain server needs sum(service);
    no server finishes the stream faster than its total work W =
    sum N^2 (steps + 1) at the best rate the GPU reaches on any size.  Also
    the share of work and of plain service time per octave of N."""
    work = np.array([float(r["n"]) ** 2 * (r["steps"] + 1) for r in reqs])
    svc = np.asarray(service, np.float64)
    octave = np.floor(np.log2([r["n"] for r in reqs])).astype(int)
    rows = []
    for o in sorted(set(octave.tolist())):
        m = octave == o
        rows.append({"n_range": [2 ** o, 2 ** (o + 1) - 1], "requests": int(m.sum()),
                     "work_share": float(work[m].sum() / work.sum()),
                     "plain_time_share": float(svc[m].sum() / svc.sum()),
                     "plain_interactions_per_s": float(work[m].sum() / svc[m].sum())})
    t_best = work.sum() / best_rate
    return {"work_interactions": float(work.sum()), "best_rate_per_s": best_rate,
            "plain_service_s": float(svc.sum()), "bound_batched_s": float(t_best),
            "speedup_bound": float(svc.sum() / t_best), "by_octave": rows}


def _pct(x, q):
    return float(np.percentile(np.asarray(x), q)) if len(x) else None


def _batched_run(reqs, eps2, dt, budget_gb, slots, work_budget=2e10, sub_work=0.0,
                 records_out=None, express_n=8192, express_ctas=32, newton3_min=16384):
    srv = BatchedServer(eps2, dt, budget_gb * 1e9, slots, work_budget=work_budget,
                        sub_work=sub_work, express_n=express_n, express_ctas=express_ctas,
                        newton3_min=newton3_min)
    recs, _, info = srv.run(reqs)
    srv.close()
    if records_out is not None:
        records_out.append({"work_budget": work_budget, "sub_work": sub_work,
                            "express_n": express_n, "records": recs})
    lat = [r["latency"] for r in recs.values() if "latency" in r]
    inter = sum(float(r["n"]) ** 2 * (r["steps"] + 1) for r in recs.values() if "latency" in r)
    span = max(r["finish"] for r in recs.values() if "finish" in r) - min(
        r["arrival"] for r in reqs)
    return {"completed": len(lat), "wall_s": info["wall_s"], "ticks": info["ticks"],
            "tick_loop_s": info["host_and_gpu_tick_s"], "systems_per_s": len(lat) / span,
            "interactions_per_s": inter / span, "latency_p50_s": _pct(lat, 50),
            "latency_p99_s": _pct(lat, 99),
            "latency_mean_s": float(np.mean(lat)) if lat else None,
            "work_budget": work_budget, "sub_work": sub_work, "express_n": express_n,
            "express_ctas": express_ctas, "newton3_min": newton3_min,
            "lanes": info.get("lanes")}


def serve_study(n_req: int = 20000, rates=(10.0,), seed: int = 5, n_lo: int = 256,
                n_hi: int = 65536, steps_lo: int = 10, steps_hi: int = 1000, dt: float = 0.005,
                eps2: float = 1e-4, budget_gb: float = 120.0, slots: int = 512,
                plain_sample: int | None = None, work_budgets=(2e10,), sub_work: float = 0.0,
                records_out=None, express_n: int = 8192, express_ctas: int = 32,
                newton3_min: int = 16384, plain_only: bool = False) -> dict:
    """Both servers on the same stream at each arrival rate.  The plain
    server's per-request service times are measured once (they do not depend
    on the arrival times) and replayed through the FIFO rule at every rate.
    The batched server runs once per work budget (interactions per tick
    above which large requests wait); the first budget is the headline.
    plain_only: the plain server alone (re-measuring it after a change to
    the single-system path; the batched server's results do not depend on
    that path)."""
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
    best = best_interaction_rate(eps2=eps2)
    out = {"study": "serving", "requests": n_req, "seed": seed, "n_range": [n_lo, n_hi],
           "steps_range": [steps_lo, steps_hi], "dt": dt, "softeningSquared": eps2,
           "budget_gb": budget_gb, "slots": slots,
           "plain_service_total_s": float(sum(service)),
           "plain_measured_requests": len(measured),
           "plain_service_predicted": len(measured) != n_req,
           "best_rates": best, "bound": throughput_bound(base, service, best["best"]),
           "by_rate": []}
    for rate in rates:
        reqs = make_requests(n_req, rate, seed, n_lo, n_hi, steps_lo, steps_hi)
        runs = [] if plain_only else [
            _batched_run(reqs, eps2, dt, budget_gb, slots, wb, sub_work, records_out,
                         express_n, express_ctas, newton3_min) for wb in work_budgets]
        arrivals = [r["arrival"] for r in reqs]
        pfin = fifo_finish_times(arrivals, service)
        plat = [f - a for f, a in zip(pfin, arrivals)]
        pspan = pfin[-1] - arrivals[0]
        p = {"systems_per_s": n_req / pspan, "latency_p50_s": _pct(plat, 50),
             "latency_p99_s": _pct(plat, 99), "latency_mean_s": float(np.mean(plat))}
        if plain_only:
            out["by_rate"].append({"rate_per_s": rate, "plain": p})
            continue
        b = runs[0]
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
    ap.add_argument("--sub-work", type=float, default=0.0,
                    help="a request takes min(8, sub_work // N^2) steps per tick (0: one)")
    ap.add_argument("--express-n", type=int, default=8192,
                    help="requests with N <= this run in the express lane (0: one lane)")
    ap.add_argument("--express-ctas", type=int, default=32,
                    help="CTA slots of the express lane's persistent force launch")
    ap.add_argument("--newton3-min", type=int, default=16384,
                    help="main-lane requests with N >= this use the Newton-3 kernel (0: none)")
    ap.add_argument("--plain-only", action="store_true",
                    help="measure and replay the plain server alone")
    ap.add_argument("--records", default=None,
                    help="write every batched request's record (JSON) to this path")
    a = ap.parse_args(argv)
    rates = [float(x) for x in a.rates.split(",")]
    budgets = [float(x) for x in a.work_budgets.split(",")]
    recs = [] if a.records else None
    r = serve_study(a.requests, rates, a.seed, a.n_lo, a.n_hi, a.steps_lo, a.steps_hi, a.dt,
                    a.eps2, a.budget_gb, a.slots, a.plain_sample, budgets, a.sub_work, recs,
                    a.express_n, a.express_ctas, a.newton3_min, a.plain_only)
    if a.records:
        with open(a.records, "w") as f:
            json.dump(recs, f)
    print(json.dumps(r))


if __name__ == "__main__":
    main()
