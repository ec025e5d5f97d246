"""Continuous batching: every result is the same alone and in the mix, and
admission respects the state budget and slot count."""
import numpy as np
import pytest

import nbody_gb300 as nb
from nbody_gb300 import serving

pytestmark = pytest.mark.gpu


def _stream(k, rate, seed):
    return serving.make_requests(k, rate, seed, n_lo=256, n_hi=6000, steps_lo=5, steps_hi=40)


def test_results_identical_alone_and_in_the_mix(cuda):
    reqs = _stream(14, 400.0, 3)
    keep = {r["id"] for r in reqs[::3]}
    srv = serving.BatchedServer(1e-4, 0.005, 4e9, 8)
    recs, mixed, info = srv.run(reqs, keep_states=keep)
    srv.close()
    assert all("latency" in r for r in recs.values())
    assert info["ticks"] > 0
    for r in reqs:
        if r["id"] not in keep:
            continue
        alone_req = dict(r, arrival=0.0)
        s = serving.BatchedServer(1e-4, 0.005, 4e9, 1)
        _, alone, _ = s.run([alone_req], keep_states={r["id"]})
        s.close()
        for a, b in zip(alone[r["id"]], mixed[r["id"]]):
            assert np.array_equal(a, b), r["id"]


def test_main_lane_results_alone_and_in_the_mix(cuda):
    """Requests above the express lane's size limit (N in [8,193, 40,000])
    run in the main lane; those with N >= 16,384 are evaluated there by the
    Newton's-third-law block-pair launch, whose per-body sums are FP64
    atomics.  One-sided systems must come out bit-identical alone and in the
    mix; Newton-3 systems repeat to FP64 summation order (an FP32
    acceleration can differ by one rounding where an FP64 sum lies on an FP32
    rounding boundary), so their states must agree to 1e-6 of their scale."""
    reqs = serving.make_requests(8, 400.0, 17, n_lo=8193, n_hi=40000, steps_lo=5,
                                 steps_hi=20)
    assert any(r["n"] >= 16384 for r in reqs) and any(r["n"] < 16384 for r in reqs)
    keep = {r["id"] for r in reqs}
    srv = serving.BatchedServer(1e-4, 0.005, 2e9, 8)
    recs, mixed, info = srv.run(reqs, keep_states=keep)
    srv.close()
    assert all("latency" in r for r in recs.values())
    assert info["lanes"]["main"]["requests"] == len(reqs)
    for r in reqs:
        s = serving.BatchedServer(1e-4, 0.005, 2e9, 1)
        _, alone, _ = s.run([dict(r, arrival=0.0)], keep_states={r["id"]})
        s.close()
        a_st, m_st = alone[r["id"]], mixed[r["id"]]
        if r["n"] < 16384:
            for a, b in zip(a_st, m_st):
                assert np.array_equal(a, b), r["id"]
        else:
            for a, b in zip(a_st[:2], m_st[:2]):  # positions, velocities
                assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max(), r["id"]


def test_tiny_budget_admits_within_limits(cuda):
    reqs = _stream(10, float("inf"), 4)
    biggest = max(r["n"] for r in reqs) * serving.BYTES_PER_BODY
    srv = serving.BatchedServer(1e-4, 0.005, budget_bytes=1.5 * biggest, max_slots=3,
                                express_n=0)  # one lane: every request in the main arena
    peak = {"bytes": 0, "slots": 0}
    orig_add = srv.ens.add

    def add(*a, **k):
        slot = orig_add(*a, **k)
        peak["bytes"] = max(peak["bytes"], srv.used_bytes + a[0].shape[0] * serving.BYTES_PER_BODY)
        peak["slots"] = max(peak["slots"], srv.ens.active())
        return slot

    srv.ens.add = add
    recs, _, _ = srv.run(reqs)
    srv.close()
    assert all("latency" in r for r in recs.values())
    assert peak["bytes"] <= 1.5 * biggest and peak["slots"] <= 3


def test_matches_plain_single_system(cuda):
    r = _stream(1, float("inf"), 9)[0]
    srv = serving.BatchedServer(1e-4, 0.005, 4e9, 2)
    _, st, _ = srv.run([r], keep_states={r["id"]})
    srv.close()
    p, v, m = serving._initial_state(r)
    s = nb.System(r["n"], nb.INTEGRATOR_KDK64, 1e-4, 0.005, 1.0)
    s.set_state64(p, v, m)
    s.step(r["steps"])
    ps, vs = s.get_state64()
    s.close()
    pe, ve, _ = st[r["id"]]
    assert np.abs(pe - ps).max() <= 1e-8 * np.abs(ps).max()
    assert np.abs(ve - vs).max() <= 1e-7 * np.abs(vs).max()


def test_express_lane_admits_within_its_limits(cuda):
    """Small requests run in the express lane, within its slot count and its
    share of the state budget; its arena runs beside the main one."""
    reqs = _stream(10, float("inf"), 4)  # N <= 6000: all express
    srv = serving.BatchedServer(1e-4, 0.005, 4e9, 8, express_slots=3)
    lane = srv.express
    assert srv.ens.max_grid() == lane.ens.max_grid()
    peak = {"bytes": 0, "slots": 0}
    orig_add = lane.ens.add

    def add(*a, **k):
        slot = orig_add(*a, **k)
        peak["bytes"] = max(peak["bytes"], lane.used_bytes + a[0].shape[0] * serving.BYTES_PER_BODY)
        peak["slots"] = max(peak["slots"], lane.ens.active())
        return slot

    lane.ens.add = add
    recs, _, info = srv.run(reqs)
    srv.close()
    assert all("latency" in r for r in recs.values())
    assert info["lanes"]["express"]["requests"] == 10 and info["lanes"]["main"]["requests"] == 0
    assert 0 < peak["slots"] <= 3 and peak["bytes"] <= lane.budget
