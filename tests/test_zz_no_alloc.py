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
# different j-splits, so they differ in rounding only)
TOL = 1e-5


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


def test_static_scratch_rejects_sizes_beyond_its_limit(cuda):
    import torch
    lib = _c_abi()
    cap = lib.nbgb_force_static_capacity_bytes()
    assert cap == 32 << 20
    nmax = cap // 16
    buf = torch.zeros((16, 4), device="cuda")
    # rejected on the host before any launch (the buffers are never touched)
    assert lib.nbgb_force_static(buf.data_ptr(), buf.data_ptr(), 1e-4, nmax + 1, None) == -7
