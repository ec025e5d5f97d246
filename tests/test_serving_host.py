"""Host logic of the serving loop (no GPU): request stream and FIFO rule."""
import math

import numpy as np

from nbody_gb300 import serving


def test_request_stream_distribution():
    reqs = serving.make_requests(20000, 10.0, 5)
    n = np.array([r["n"] for r in reqs])
    steps = np.array([r["steps"] for r in reqs])
    arr = np.array([r["arrival"] for r in reqs])
    assert n.min() >= 256 and n.max() <= 65536
    # log-uniform: median near sqrt(256 * 65536) = 4096
    assert abs(math.log(np.median(n)) - math.log(4096)) < 0.1
    assert steps.min() >= 10 and steps.max() <= 1000 and abs(steps.mean() - 505) < 10
    gaps = np.diff(np.concatenate([[0.0], arr]))
    assert abs(gaps.mean() - 0.1) < 0.005 and np.all(gaps >= 0)  # Poisson, rate 10/s
    assert len({r["seed"] for r in reqs}) == 20000
    assert serving.make_requests(20000, 10.0, 5) == reqs  # seeded


def test_fifo_finish_times():
    # server idle until an arrival, then busy back to back
    f = serving.fifo_finish_times([0.0, 0.5, 0.6, 10.0], [1.0, 1.0, 1.0, 2.0])
    assert f == [1.0, 2.0, 3.0, 12.0]


def test_all_at_once_stream():
    reqs = serving.make_requests(10, float("inf"), 1)
    assert all(r["arrival"] == 0.0 for r in reqs)


class FakeEnsemble:
    """Host stand-in for nbgb_ensemble with the same tick semantics: a new
    system's first tick computes its initial forces, each later tick moves it
    min(sub, steps left) steps; finished = started with no steps left."""

    def __init__(self, max_bodies, max_systems, eps2):
        self.max_bodies, self.max_systems = max_bodies, max_systems
        self.grid = self.grid_max = 304
        self.sys = {}
        self.events = []  # (tick count, "add"/"remove", slot, n)
        self.ticks = 0
        self.peak_active = 0
        self.peak_bodies = 0

    def max_grid(self):
        return self.grid_max

    def set_grid(self, ctas):
        assert 0 < ctas <= self.grid_max
        self.grid = ctas

    def set_newton3_min(self, nmin):
        self.newton3_min = nmin

    def set_priority(self, high):
        self.high_priority = bool(high)

    def add(self, p, v, m, dt, steps):
        free = [s for s in range(self.max_systems) if s not in self.sys]
        bodies = sum(x["n"] for x in self.sys.values()) + p.shape[0]
        if not free or bodies > self.max_bodies:
            return None
        slot = free[0]
        self.sys[slot] = {"n": p.shape[0], "left": steps, "started": False, "sub": 1}
        self.events.append((self.ticks, "add", slot, p.shape[0]))
        self.peak_active = max(self.peak_active, len(self.sys))
        self.peak_bodies = max(self.peak_bodies, bodies)
        return slot

    def set_substeps(self, slot, sub):
        assert 1 <= sub <= 8
        self.sys[slot]["sub"] = sub

    def tick(self, k=1):
        for _ in range(k):
            self.ticks += 1
            for x in self.sys.values():
                if not x["started"]:
                    x["started"] = True
                elif x["left"] > 0:
                    x["left"] -= min(x["sub"], x["left"])

    def synchronize(self):
        pass

    def finished(self, max_n=65536):
        return [s for s, x in self.sys.items() if x["started"] and x["left"] == 0][:max_n]

    def get_state(self, slot):
        n = self.sys[slot]["n"]
        return np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 4), np.float32)

    def remove(self, slot):
        self.events.append((self.ticks, "remove", slot, self.sys[slot]["n"]))
        del self.sys[slot]

    def active(self):
        return len(self.sys)

    def close(self):
        pass


def _server(**kw):
    return serving.BatchedServer(1e-4, 0.005, ensemble_factory=FakeEnsemble, **kw)


def _reqs(ns, steps=20):
    return [{"id": i, "n": n, "steps": steps, "seed": 100 + i, "arrival": 0.0}
            for i, n in enumerate(ns)]


def test_lanes_route_by_size():
    srv = _server(budget_bytes=4e9, express_n=1000, express_ctas=32)
    assert srv.ens.grid == 304 - 32 and srv.express.ens.grid == 32
    assert srv.express.ens.high_priority and srv.ens.newton3_min == 16384
    reqs = _reqs([300, 5000, 800, 2000, 1000, 1001])
    recs, _, info = srv.run(reqs)
    assert all("latency" in r for r in recs.values())
    assert info["lanes"]["express"]["requests"] == 3 and info["lanes"]["main"]["requests"] == 3
    assert sorted(e[3] for e in srv.express.ens.events if e[1] == "add") == [300, 800, 1000]
    assert srv.used_bytes == 0  # every request retired


def test_large_requests_first_come_first_served():
    # budget for one large request at a time: later (even smaller) large
    # requests must not overtake a waiting one
    ns = [3000, 20000, 12000, 15000, 11000]
    srv = _server(budget_bytes=4e9, express_n=0, work_budget=1.0, small_work=1e6)
    recs, _, _ = srv.run(_reqs(ns))
    admits = [recs[i]["admit"] for i in range(len(ns))]
    assert admits == sorted(admits)
    adds = [e for e in srv.ens.events if e[1] == "add"]
    assert [e[3] for e in adds] == ns
    # one large request at a time: each add comes after the previous remove
    removes = [e for e in srv.ens.events if e[1] == "remove"]
    for k in range(1, len(adds)):
        assert adds[k][0] >= removes[k - 1][0]


def test_small_requests_join_past_the_work_budget():
    ns = [20000, 30000, 500, 600, 700]
    srv = _server(budget_bytes=4e9, express_n=0, work_budget=1.0, small_work=1e6)
    recs, _, _ = srv.run(_reqs(ns))
    first_large_done = recs[0]["finish"]
    for i in (2, 3, 4):  # small: admitted while the first large one runs
        assert recs[i]["admit"] <= first_large_done
    assert recs[1]["admit"] >= first_large_done  # the second large one waited


def test_slot_and_byte_limits():
    ns = [4000] * 12
    budget = 3.5 * 4000 * serving.BYTES_PER_BODY
    srv = _server(budget_bytes=budget, max_slots=5, express_n=0)
    recs, _, _ = srv.run(_reqs(ns))
    assert all("latency" in r for r in recs.values())
    assert srv.ens.peak_active <= 3  # the byte budget binds before the slots
    srv = _server(budget_bytes=4e9, max_slots=2, express_n=0)
    srv.run(_reqs(ns))
    assert srv.ens.peak_active <= 2


def test_substeps_ticks():
    # one request alone: 1 initial-force tick + ceil(steps / sub) ticks
    for n, steps in ((300, 20), (300, 21), (5000, 20)):
        srv = _server(budget_bytes=4e9, express_n=0, sub_work=4e8)
        sub = srv.main._sub(n)
        _, _, info = srv.run(_reqs([n], steps))
        assert info["ticks"] == 1 + -(-steps // sub), (n, steps, sub)
        assert sub == min(8, int(4e8 // n ** 2)) or sub == 1
