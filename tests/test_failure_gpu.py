"""Failure handling without a GPU fault: a bounded wait runs out on purpose
(an mbarrier nothing completes, 20 ms limit), the kernel reports it in the
device status word and returns, and the context stays usable."""
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_reports(cuda):
    import torch
    bits = nb.load().nbgb_selftest_bounded_wait(20.0)
    assert bits == 0x1  # NBGB_STATUS_WAIT_TIMEOUT
    assert nb.last_status() == 0  # read and cleared
    # the context is still usable: a force pass after it is correct
    pm, _ = nb.ic_uniform_ball(3000, 5)
    out = nb.force(torch.from_numpy(pm).cuda(), 1e-4).cpu().numpy()
    assert O.per_body_rel_error(out, O.ieee().forces_aos(pm, 1e-4))[0] <= 1e-5
    assert nb.last_status() == 0


def test_selftest_rejects_bad_limits(cuda):
    assert nb.load().nbgb_selftest_bounded_wait(0.0) == -1
    assert nb.load().nbgb_selftest_bounded_wait(5000.0) == -1
