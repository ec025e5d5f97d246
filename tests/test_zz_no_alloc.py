"""The allocation-free entry point nbgb_force_static, called through the C ABI.

It exists for callers that cannot allocate device memory at run time (hosts
that own all device memory through a pool or a fixed budget, and
latency-critical loops where cudaMalloc may synchronise the device).  Its
scratch is a fixed device array inside the library, shared by every call, so
this test makes two calls in a row and checks both against the ordinary
nbgb_force entry point, within the force tolerance the other tests use.  It
runs last (file name) and also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import nbody_gb300 as nb
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# per-body |dF|/|F| between two evaluations of the same sum (they may use
# different j-splits, so they differ in rounding only), and against the FP64
# all-pairs sum (the gate of the other force tests)
TOL = 1e-5
TOL_VS_FP64 = 5e-6


def _c_abi():
    lib = ctypes.CDLL(nb.LIB_PATH)
    lib.nbgb_force_static.restype = ctypes.c_int
    lib.nbgb_force_static.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float,
                                      ctypes.c_size_t, ctypes.c_void_p]
    lib.nbgb_force_static_capacity_bytes.restype = ctypes.c_size_t
    lib.nbgb_force.restype = ctypes.c_int
    lib.nbgb_force.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_size_t,
                               ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    lib.nbgb_force_workspace_bytes.restype = ctypes.c_size_t
    lib.nbgb_force_workspace_bytes.argtypes = [ctypes.c_size_t]
    return lib


@pytest.mark.parametrize("n", [16384, 100003])
def test_static_scratch_matches_allocating_entry_twice(cuda, n):
    import torch
    lib = _c_abi()
    stream = torch.cuda.current_stream().cuda_stream
    _, _, pm_np, _ = nb.ic_plummer(n, 77 + n)
    pm = torch.from_numpy(pm_np).cuda()

    wsb = lib.nbgb_force_workspace_bytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    ref = torch.empty_like(pm)
    assert lib.nbgb_force(ref.data_ptr(), pm.data_ptr(), 1e-4, n, ws.data_ptr(), wsb,
                          stream) == 0

    outs = []
    for _ in range(2):  # the second call reuses the array the first one left
        out = torch.full_like(pm, float("nan"))
        assert lib.nbgb_force_static(out.data_ptr(), pm.data_ptr(), 1e-4, n, stream) == 0
        outs.append(out)
    torch.cuda.synchronize()
    assert nb.last_status() == 0
    r = ref.cpu().numpy()
    for out in outs:
        o = out.cpu().numpy()
        assert np.all(np.isfinite(o))
        assert O.per_body_rel_error(o, r)[0] <= TOL
    assert np.array_equal(outs[0].cpu().numpy(), outs[1].cpu().numpy())


def test_static_scratch_against_fp64_and_across_sizes(cuda):
    """The same array serves calls of different sizes and plans in turn: a
    100,003-body call (j-split partials and counters in use) followed by a
    16,384-body call, each checked against the allocating entry point and
    the FP64 all-pairs sum on a sample of bodies."""
    import torch
    lib = _c_abi()
    stream = torch.cuda.current_stream().cuda_stream
    for n in (100003, 16384, 100003):
        _, _, pm_np, _ = nb.ic_plummer(n, 5 + n)
        pm = torch.from_numpy(pm_np).cuda()
        out = torch.full_like(pm, float("nan"))
        assert lib.nbgb_force_static(out.data_ptr(), pm.data_ptr(), 1e-4, n, stream) == 0
        wsb = lib.nbgb_force_workspace_bytes(n)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        ref = torch.empty_like(pm)
        assert lib.nbgb_force(ref.data_ptr(), pm.data_ptr(), 1e-4, n, ws.data_ptr(), wsb,
                              stream) == 0
        torch.cuda.synchronize()
        assert nb.last_status() == 0
        o = out.cpu().numpy()
        assert O.per_body_rel_error(o, ref.cpu().numpy())[0] <= TOL
        idx = np.random.default_rng(n).choice(n, 256, replace=False)
        f64 = O.ieee().forces_f64(pm_np, float(np.float32(1e-4)), idx)
        t = np.zeros((idx.size, 4))
        t[:, :3] = f64
        assert O.per_body_rel_error(o[idx], t)[0] <= TOL_VS_FP64


@pytest.mark.parametrize("delta", [0, 1])
def test_static_scratch_at_its_documented_limit(cuda, delta):
    """N = capacity / 16 (and one less, padded to the same tiles) is accepted
    and evaluated; spot checks against the allocating entry point."""
    import torch
    lib = _c_abi()
    n = lib.nbgb_force_static_capacity_bytes() // 16 - delta
    stream = torch.cuda.current_stream().cuda_stream
    _, _, pm_np, _ = nb.ic_plummer(n, 99)
    pm = torch.from_numpy(pm_np).cuda()
    out = torch.full_like(pm, float("nan"))
    assert lib.nbgb_force_static(out.data_ptr(), pm.data_ptr(), 1e-4, n, stream) == 0
    wsb = lib.nbgb_force_workspace_bytes(n)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    ref = torch.empty_like(pm)
    assert lib.nbgb_force(ref.data_ptr(), pm.data_ptr(), 1e-4, n, ws.data_ptr(), wsb,
                          stream) == 0
    torch.cuda.synchronize()
    assert nb.last_status() == 0
    o = out.cpu().numpy()
    assert np.all(np.isfinite(o))
    idx = np.random.default_rng(3).choice(n, 4096, replace=False)
    assert O.per_body_rel_error(o[idx], ref.cpu().numpy()[idx])[0] <= TOL


def test_static_scratch_rejects_sizes_beyond_its_limit(cuda):
    import torch
    lib = _c_abi()
    cap = lib.nbgb_force_static_capacity_bytes()
    assert cap == 32 << 20
    nmax = cap // 16
    buf = torch.zeros((16, 4), device="cuda")
    # rejected on the host before any launch (the buffers are never touched)
    assert lib.nbgb_force_static(buf.data_ptr(), buf.data_ptr(), 1e-4, nmax + 1, None) == -7
