"""ctypes binding of libnbody_gb300.so (the C ABI in include/nbody_gb300.h).

The library is built in-tree by nbody_gb300/build.py.  There is no fallback:
if the shared object is missing or fails to load, every call raises.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libnbody_gb300.so")

c_f32p = ctypes.POINTER(ctypes.c_float)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_i64p = ctypes.POINTER(ctypes.c_longlong)
c_intp = ctypes.POINTER(ctypes.c_int)
c_sizep = ctypes.POINTER(ctypes.c_size_t)
c_vp = ctypes.c_void_p
c_size = ctypes.c_size_t

# name: (restype, argtypes)
SIGNATURES = {
    "ComputeGravitation_GPU_GB300": (ctypes.c_float, [c_vp, c_vp, ctypes.c_float, c_size]),
    "ComputeGravitation_GPU_GB300_Newton3": (ctypes.c_float, [c_vp, c_vp, ctypes.c_float,
                                                              c_size]),
    "nbgb_release_workspace": (None, []),
    "nbgb_force_workspace_bytes": (c_size, [c_size]),
    "nbgb_force": (ctypes.c_int, [c_vp, c_vp, ctypes.c_float, c_size, c_vp, c_size, c_vp]),
    "nbgb_force_ex": (ctypes.c_int, [c_vp, c_vp, ctypes.c_float, c_size, c_vp, c_size,
                                     ctypes.c_int, ctypes.c_int, c_vp]),
    "nbgb_force_newton3_workspace_bytes": (c_size, [c_size]),
    "nbgb_force_newton3": (ctypes.c_int, [c_vp, c_vp, ctypes.c_float, c_size, c_vp, c_size,
                                          c_vp]),
    "nbgb_force_plan": (ctypes.c_int, [c_size, ctypes.c_int, ctypes.c_int, c_intp, c_intp,
                                       c_sizep]),
    "nbgb_force_plan_on": (ctypes.c_int, [c_size, ctypes.c_int, c_intp, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, c_intp, c_intp, c_intp,
                                          c_sizep]),
    "nbgb_force_device_info": (ctypes.c_int, [c_intp, c_intp, ctypes.c_int]),
    "nbgb_force_num_configs": (ctypes.c_int, []),
    "nbgb_force_config_name": (ctypes.c_char_p, [ctypes.c_int]),
    "nbgb_force_set_speed": (ctypes.c_int, [ctypes.c_int, ctypes.c_double]),
    "nbgb_force_get_speed": (ctypes.c_double, [ctypes.c_int]),
    "nbgb_force_rows_workspace_bytes": (c_size, [c_size, c_size]),
    "nbgb_force_rows": (ctypes.c_int, [c_vp, c_vp, ctypes.c_float, c_size, c_size, c_size, c_vp,
                                       c_size, c_vp]),
    "nbgb_force_static": (ctypes.c_int, [c_vp, c_vp, ctypes.c_float, c_size, c_vp]),
    "nbgb_force_static_capacity_bytes": (c_size, []),
    "nbgb_integrate_reference": (ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_float,
                                                ctypes.c_float, c_size, c_vp]),
    "nbgb_integrate_reference_ex": (ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_float,
                                                   ctypes.c_float, c_size, ctypes.c_int, c_vp]),
    "nbgb_system_create": (c_vp, [c_size, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float]),
    "nbgb_system_destroy": (None, [c_vp]),
    "nbgb_system_set_state": (ctypes.c_int, [c_vp, c_f32p, c_f32p]),
    "nbgb_system_set_state64": (ctypes.c_int, [c_vp, c_f64p, c_f64p, c_f32p]),
    "nbgb_system_step": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_system_set_graph": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_system_set_force_algorithm": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_system_synchronize": (ctypes.c_int, [c_vp]),
    "nbgb_system_set_timing": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_system_last_force_ms": (ctypes.c_int, [c_vp, c_f32p]),
    "nbgb_system_last_integrate_ms": (ctypes.c_int, [c_vp, c_f32p, c_f32p]),
    "nbgb_system_sync_velocities": (ctypes.c_int, [c_vp]),
    "nbgb_system_get_state": (ctypes.c_int, [c_vp, c_f32p, c_f32p]),
    "nbgb_system_get_state64": (ctypes.c_int, [c_vp, c_f64p, c_f64p]),
    "nbgb_system_get_force": (ctypes.c_int, [c_vp, c_f32p]),
    "nbgb_system_diagnostics": (ctypes.c_int, [c_vp, c_f64p]),
    "nbgb_system_device_posmass": (c_vp, [c_vp]),
    "nbgb_system_device_force": (c_vp, [c_vp]),
    "nbgb_system_stream": (c_vp, [c_vp]),
    "nbgb_system_plan": (ctypes.c_int, [c_vp, c_intp, c_intp]),
    "nbgb_system_set_plan": (ctypes.c_int, [c_vp, ctypes.c_int, ctypes.c_int]),
    "nbgb_ensemble_create": (c_vp, [c_size, ctypes.c_int, ctypes.c_float]),
    "nbgb_ensemble_destroy": (None, [c_vp]),
    "nbgb_ensemble_device_bytes": (c_size, [c_vp]),
    "nbgb_ensemble_set_bucket_plan": (ctypes.c_int, [c_vp, ctypes.c_int, ctypes.c_int,
                                                     ctypes.c_int, ctypes.c_int]),
    "nbgb_ensemble_add": (ctypes.c_int, [c_vp, c_f64p, c_f64p, c_f32p, c_size, ctypes.c_double,
                                         ctypes.c_longlong, c_intp]),
    "nbgb_ensemble_tick": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_ensemble_set_graph": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_ensemble_synchronize": (ctypes.c_int, [c_vp]),
    "nbgb_ensemble_finished": (ctypes.c_int, [c_vp, c_intp, ctypes.c_int]),
    "nbgb_ensemble_get_state": (ctypes.c_int, [c_vp, ctypes.c_int, c_f64p, c_f64p, c_f32p]),
    "nbgb_ensemble_slot_info": (ctypes.c_int, [c_vp, ctypes.c_int, c_i64p]),
    "nbgb_ensemble_remove": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_ensemble_set_substeps": (ctypes.c_int, [c_vp, ctypes.c_int, ctypes.c_int]),
    "nbgb_ensemble_set_grid": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_ensemble_max_grid": (ctypes.c_int, [c_vp]),
    "nbgb_ensemble_set_newton3_min": (ctypes.c_int, [c_vp, ctypes.c_size_t]),
    "nbgb_ensemble_set_priority": (ctypes.c_int, [c_vp, ctypes.c_int]),
    "nbgb_ensemble_active": (ctypes.c_int, [c_vp]),
    "nbgb_ensemble_stream": (c_vp, [c_vp]),
    "nbgb_ic_reference": (ctypes.c_int, [c_f32p, c_f32p, c_size, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_uint]),
    "nbgb_ic_uniform_ball": (ctypes.c_int, [c_f32p, c_f32p, c_size, ctypes.c_double,
                                            ctypes.c_double, ctypes.c_double,
                                            ctypes.c_ulonglong]),
    "nbgb_ic_plummer": (ctypes.c_int, [c_f64p, c_f64p, c_f32p, c_f32p, c_size,
                                       ctypes.c_ulonglong]),
    "nbgb_force_f64_host": (ctypes.c_int, [c_f32p, c_size, ctypes.c_double, c_i64p, c_size,
                                           c_f64p, c_f64p]),
    "nbgb_crosscheck_max_rel_error": (ctypes.c_float, [c_f32p, c_f32p, c_size]),
    "nbgb_force_error_stats": (ctypes.c_int, [c_f32p, c_f64p, c_i64p, c_size, c_f64p, c_f64p]),
    "nbgb_measure_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_f64p,
                                         c_f32p]),
    "nbgb_measure_copy": (ctypes.c_int, [c_size, ctypes.c_int, c_f64p, c_f32p]),
    "nbgb_last_status": (ctypes.c_int, []),
    "nbgb_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "nbgb_version": (ctypes.c_char_p, []),
    "nbgb_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_double]),
    "nbgb_selftest_conversions": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_ulonglong,
                                                 ctypes.POINTER(ctypes.c_ulonglong)]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load the in-tree library once; raise loudly if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -m nbody_gb300.build` "
            "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class NbgbError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = load().nbgb_status_string(code).decode()
        super().__init__(f"{where}: {msg} (code {code})")
        self.code = code


def check(code: int, where: str) -> None:
    if code != 0:
        raise NbgbError(code, where)
