"""The GPU integrator in reference mode is bit-identical to integrateOne
(src/nbody.cu:158-182) evaluated in IEEE binary32 by the oracle."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu


def test_integrate_reference_bit_exact_random(cuda):
    import torch
    rng = np.random.default_rng(5)
    n = 100003
    pm = rng.normal(size=(n, 4)).astype(np.float32)
    vm = rng.normal(size=(n, 4)).astype(np.float32)
    vm[:, 3] = rng.uniform(1, 20000, n).astype(np.float32)
    f = rng.normal(size=(n, 4)).astype(np.float32)
    tp, tv, tf = (torch.from_numpy(a.copy()).cuda() for a in (pm, vm, f))
    nb.integrate_reference(tp, tv, tf, 0.016, 0.95)
    torch.cuda.synchronize()
    O.ieee().integrate(pm, vm, f, 0.016, 0.95)
    assert np.array_equal(tp.cpu().numpy(), pm)
    assert np.array_equal(tv.cpu().numpy(), vm)


def test_integrate_reference_reproduces_golden_step(cuda):
    import torch
    t = golden("traj1024")
    tp = torch.from_numpy(t["posMass0"]).cuda()
    tv = torch.from_numpy(t["velInvMass0"]).cuda()
    tf = torch.from_numpy(t["force_step1"]).cuda()
    nb.integrate_reference(tp, tv, tf, float(t["dt"]), float(t["damping"]))
    torch.cuda.synchronize()
    assert np.array_equal(tp.cpu().numpy(), t["posMass1"])
    assert np.array_equal(tv.cpu().numpy(), t["velInvMass1"])
