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
