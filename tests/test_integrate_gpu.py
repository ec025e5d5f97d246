"""The GPU integrator in reference mode is bit-identical to integrateOne
(src/nbody.cu:158-182) evaluated in IEEE binary32 by the oracle."""
import ctypes

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


@pytest.mark.parametrize("n", [1001, 4096])
def test_kdk_step_is_the_fp64_leapfrog(cuda, n):
    """One FP64 kick-drift-kick step on the GPU (kick+drift kernel, force pass,
    half-kick kernel) against the same leapfrog evaluated on the host in FP64
    with the GPU's own accelerations: equal to FP64 rounding (the GPU fuses
    each update into one multiply-add).  The FP32 posMass the next force pass
    reads is the FP64 position rounded, with the mass; odd N covers the
    kernels' last, half-filled body pair."""
    import torch
    p, v, pm, _ = nb.ic_plummer(n, 31)
    m = pm[:, 3].copy()
    dt = float(np.float32(0.005))  # the system keeps dt in binary32
    # the system's first force pass uses the same plan as nb.force: same bits
    a0 = nb.force(torch.from_numpy(pm).cuda(), 1e-4).cpu().numpy()[:, :3].astype(np.float64)
    s = nb.System(n, nb.INTEGRATOR_KDK64, 1e-4, dt, 1.0)
    s.set_state64(p, v, m)
    s.step(1)
    p1, v1 = s.get_state64()
    a1 = s.get_force()[:, :3].astype(np.float64)
    pm1, _ = s.get_state()
    s.close()
    vh = v + a0 * (0.5 * dt)
    xe = p + vh * dt
    ve = vh + a1 * (0.5 * dt)
    assert np.allclose(p1, xe, rtol=1e-14, atol=1e-16)
    assert np.allclose(v1, ve, rtol=1e-14, atol=1e-16)
    assert np.array_equal(pm1[:, :3], p1.astype(np.float32))
    assert np.array_equal(pm1[:, 3], m)


def test_integer_pipe_conversions_equal_hardware(cuda):
    """The FP64 integrate kernels convert binary32 <-> binary64 with integer
    operations (GB300's FP64 pipe is narrow); on 2^24 random bit patterns of
    every class, half of them near the fast paths' exponent limits, every
    result equals the hardware conversion's."""
    bad = ctypes.c_ulonglong(99)
    assert nb.load().nbgb_selftest_conversions(1 << 24, 12345, ctypes.byref(bad)) == 0
    assert bad.value == 0
