"""Same-box comparison with the reference's own GPU kernels.

oracle/Makefile (target refgpu, run where the reference sources are present)
compiles src/nbody_GPU_AOS.cu, src/nbody_GPU_Shared.cu and
src/nbody_GPU_Shuffle.cu unchanged into sm_103a cubins under oracle/_ref/;
oracle/refgpu_launch.c launches them with the reference's own grid
(<<<300, 256>>>).  This test checks their forces against ours (both GPU
implementations of the same sum) and prints both timings; it is skipped where
the cubins were not built.  The reference kernels assume N % 1024 == 0
(src/nbody.cu:967), which every size here satisfies.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import oracle as O

import nbody_gb300 as nb

pytestmark = pytest.mark.gpu

REF = os.path.join(ROOT, "oracle", "_ref")
LAUNCHER = os.path.join(ROOT, "oracle", "_build", "librefgpu.so")
# kernel name (C++ mangled, as nm prints the host declaration), launch shape
KERNELS = {
    "GPU_AOS": ("_Z31ComputeNBodyGravitation_GPU_AOSIfEvPT_S1_mS0_", 0, 1),
    "GPU_Shared": ("_Z30ComputeNBodyGravitation_SharedPfS_fm", 256 * 16, 0),
    "GPU_Shuffle": ("_Z31ComputeNBodyGravitation_ShufflePfS_fm", 0, 0),
}


def _launcher():
    if not all(os.path.exists(os.path.join(REF, f"{k}.cubin")) for k in KERNELS):
        pytest.skip("reference GPU cubins not built here (make -C oracle refgpu)")
    lib = ctypes.CDLL(LAUNCHER)
    lib.refgpu_time.restype = ctypes.c_double
    lib.refgpu_time.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint,
                                ctypes.c_uint, ctypes.c_ulonglong, ctypes.c_ulonglong,
                                ctypes.c_float, ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    return lib


def _ref_run(lib, name, force, pm, eps2, n, reps):
    sym, shmem, order = KERNELS[name]
    ms = lib.refgpu_time(os.path.join(REF, f"{name}.cubin").encode(), sym.encode(), 300, 256,
                         shmem, force.data_ptr(), pm.data_ptr(), eps2, n, order, reps)
    assert ms > 0, f"{name}: CUDA driver error {-ms}"
    return ms


def test_reference_gpu_kernels_agree_and_are_slower(cuda):
    import torch
    lib = _launcher()
    results = {}
    for n, reps in ((16384, 20), (262144, 2)):
        _, _, pm_np, _ = nb.ic_plummer(n, 1234)
        pm = torch.from_numpy(pm_np).cuda()
        idx = np.random.default_rng(n).choice(n, 512, replace=False)
        f64 = O.ieee().forces_f64(pm_np, float(np.float32(1e-4)), idx)
        ours = nb.force(pm, 1e-4)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            nb.force(pm, 1e-4, out=ours)
        e1.record()
        torch.cuda.synchronize()
        ours_ms = e0.elapsed_time(e1) / reps
        err = {"GB300 (this library)": nb.force_error_stats(ours.cpu().numpy(), f64, idx)}
        row = {"GB300 (this library)": ours_ms}
        for name in KERNELS:
            f = torch.zeros_like(pm)
            row[f"reference {name}"] = _ref_run(lib, name, f, pm, 1e-4, n, reps)
            err[f"reference {name}"] = nb.force_error_stats(f.cpu().numpy(), f64, idx)
        results[n] = {k: {"ms": v, "G_interactions_per_s": n * n / v / 1e6,
                          "max_rel_err_vs_fp64": err[k][0], "rms_rel_err_vs_fp64": err[k][1]}
                      for k, v in row.items()}
        assert err["GB300 (this library)"][0] <= 5e-6
        for k, (mx, _) in err.items():
            assert mx <= 1e-4, k  # every kernel computes the same sum
        fastest_ref = min(v for k, v in row.items() if k.startswith("reference"))
        assert ours_ms < fastest_ref
    print("\nREF_GPU_COMPARISON " + json.dumps(results))
