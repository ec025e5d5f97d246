"""GB300 (sm_103a) all-pairs softened gravity: Python mirror of the C ABI.

The reference (tycho/nbody) exposes its force path as rows of an algorithm
table, `float (*)(float *force, float *posMass, float softeningSquared,
size_t N)` (src/nbody.h:68), driven once per step by ComputeGravitation()
(src/nbody.cu:293-470), which integrates on the host with integrateOne
(src/nbody.cu:158-182).  This package keeps those names and meanings:

  ComputeGravitation_GPU_GB300(force, posMass, softeningSquared, N) -> ms
      the drop-in algorithm row (device pointers, returns ms, 0 on error)
  force(posMass, softeningSquared)          stream-ordered force on tensors
  integrate_reference(posMass, velInvMass, force, dt, damping)
      integrateOne on the GPU, bit-identical to its IEEE binary32 evaluation
  System(N, ...)                            device-resident step loop
  ic_reference / ic_uniform_ball / ic_plummer   initial conditions
  crosscheck_max_rel_error                  the reference's crosscheck metric

All compute runs in libnbody_gb300.so; there is no CPU fallback.  PyTorch is
used only for device memory and streams.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import LIB_PATH, NbgbError, check, load  # noqa: F401

INTEGRATOR_REFERENCE = 0
INTEGRATOR_KDK64 = 1
INTEGRATOR_REFERENCE_FUSED = 2  # x = fma(v, dt, x), as the reference binary computes it

# Reference driver constants (src/nbody.cu:80-81, 151-156).
REFERENCE_SOFTENING = 0.1
REFERENCE_DAMPING = 0.95
REFERENCE_TIMESTEP = 0.016
REFERENCE_SCALE = 0.9
REFERENCE_VELOCITY_SCALE = 8.0
REFERENCE_SEED = 7
# FLOP per interaction in the reference's GFLOPS figure (src/nbody.cu:1027).
FLOPS_PER_INTERACTION = 20


def _torch():
    import torch
    return torch


def _f32p(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _f64p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _dev(t) -> int:
    """Device address of a CUDA tensor (or an int address)."""
    if isinstance(t, int):
        return t
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _stream(stream) -> int:
    if stream is None:
        return _torch().cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


# ---------------------------------------------------------------------------
# Drop-in algorithm row
# ---------------------------------------------------------------------------
def ComputeGravitation_GPU_GB300(force, posMass, softeningSquared: float, N: int) -> float:
    """The reference's AOS algorithm signature: device buffers in, elapsed
    milliseconds out (0.0 means failure / skip, src/nbody.cu:385-386)."""
    return float(load().ComputeGravitation_GPU_GB300(_dev(force), _dev(posMass),
                                                     softeningSquared, N))


def ComputeGravitation_GPU_GB300_Newton3(force, posMass, softeningSquared: float, N: int) -> float:
    """The Newton's-third-law variant as a table row (same conventions)."""
    return float(load().ComputeGravitation_GPU_GB300_Newton3(_dev(force), _dev(posMass),
                                                            softeningSquared, N))


def release_workspace() -> None:
    load().nbgb_release_workspace()


# ---------------------------------------------------------------------------
# Stream-ordered force
# ---------------------------------------------------------------------------
def force_plan(N: int, config: int = -1, nsplit: int = -1):
    """(configuration, slice count, workspace bytes) of the plan nbgb_force
    runs for N (config / nsplit as for force())."""
    c, s, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
    check(load().nbgb_force_plan(N, config, nsplit, ctypes.byref(c), ctypes.byref(s),
                                 ctypes.byref(w)), "nbgb_force_plan")
    return c.value, s.value, w.value


def force_plan_on(N: int, sms: int, occupancy, config: int = -1, nsplit: int = -1):
    """The planner's decision for N on a device with `sms` SMs and
    occupancy[c] resident CTAs per SM of configuration c, without a GPU:
    (configuration, slice count, whole i-blocks, workspace bytes)."""
    lib = load()
    occ = (ctypes.c_int * len(occupancy))(*[int(x) for x in occupancy])
    c, s, f, w = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
    check(lib.nbgb_force_plan_on(N, sms, occ, len(occupancy), config, nsplit, ctypes.byref(c),
                                 ctypes.byref(s), ctypes.byref(f), ctypes.byref(w)),
          "nbgb_force_plan_on")
    return c.value, s.value, f.value, w.value


def force_device_info():
    """(SM count, resident CTAs per SM of every configuration) of the current
    device, as the planner sees them."""
    lib = load()
    n = lib.nbgb_force_num_configs()
    occ = (ctypes.c_int * n)()
    sms = ctypes.c_int()
    check(lib.nbgb_force_device_info(ctypes.byref(sms), occ, n), "nbgb_force_device_info")
    return sms.value, list(occ)


def force_config_names():
    lib = load()
    return [lib.nbgb_force_config_name(i).decode() for i in range(lib.nbgb_force_num_configs())]


class Workspace:
    """Device scratch for force(); grows on demand (a torch byte tensor)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int):
        torch = _torch()
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device="cuda")
        return self.buf


_default_ws = Workspace()


def force(posMass, softeningSquared: float, out=None, stream=None, workspace: Workspace = None,
          config: int = -1, nsplit: int = -1):
    """F_i = sum_j m_j d_ij / (|d_ij|^2 + eps2)^1.5 for a (N,4) float32 CUDA
    tensor {x,y,z,m}; returns (N,4) {fx,fy,fz,0}.  config / nsplit force a
    plan (-1: the planner's choice; nsplit > 0 splits every i-block's
    sources nsplit ways, nsplit <= -2 only the i-blocks left over after
    whole rounds of CTA slots, -nsplit ways)."""
    torch = _torch()
    n = posMass.shape[0]
    if out is None:
        out = torch.empty((n, 4), dtype=torch.float32, device=posMass.device)
    if n == 0:
        return out
    _, _, wsb = force_plan(n, config, nsplit)
    ws = (workspace or _default_ws).get(wsb)
    check(load().nbgb_force_ex(_dev(out), _dev(posMass), softeningSquared, n, ws.data_ptr(),
                               ws.numel(), config, nsplit, _stream(stream)), "nbgb_force")
    return out


def force_rows(posMass, softeningSquared: float, row_begin: int, row_end: int, out=None,
               stream=None, workspace: Workspace = None):
    """Forces on the target rows [row_begin, row_end) of a (N,4) float32
    CUDA tensor against all N sources (one rank's share of a row-sharded
    evaluation, src/nbody_multiGPU.cu:47-125); returns (rows,4)."""
    torch = _torch()
    n = posMass.shape[0]
    rows = row_end - row_begin
    if out is None:
        out = torch.empty((max(rows, 0), 4), dtype=torch.float32, device=posMass.device)
    if rows <= 0:
        return out
    lib = load()
    wsb = lib.nbgb_force_rows_workspace_bytes(n, rows)
    if wsb == 0:
        raise NbgbError(-1, "nbgb_force_rows_workspace_bytes")
    ws = (workspace or _default_ws).get(wsb)
    check(lib.nbgb_force_rows(_dev(out), _dev(posMass), softeningSquared, n, row_begin, row_end,
                              ws.data_ptr(), ws.numel(), _stream(stream)), "nbgb_force_rows")
    return out


def force_newton3(posMass, softeningSquared: float, out=None, stream=None,
                  workspace: Workspace = None):
    """Same sum as force(), each pair evaluated once (Newton's third law)."""
    torch = _torch()
    n = posMass.shape[0]
    if out is None:
        out = torch.empty((n, 4), dtype=torch.float32, device=posMass.device)
    if n == 0:
        return out
    lib = load()
    wsb = lib.nbgb_force_newton3_workspace_bytes(n)
    ws = (workspace or _default_ws).get(wsb)
    check(lib.nbgb_force_newton3(_dev(out), _dev(posMass), softeningSquared, n, ws.data_ptr(),
                                 ws.numel(), _stream(stream)), "nbgb_force_newton3")
    return out


def integrate_reference(posMass, velInvMass, force_, dt: float, damping: float, stream=None,
                        fused_drift: bool = False):
    """In place on (N,4) float32 CUDA tensors (src/nbody.cu:158-182); with
    fused_drift the position update is one fused multiply-add, as the
    reference binary built with its own flags computes it."""
    n = posMass.shape[0]
    check(load().nbgb_integrate_reference_ex(_dev(posMass), _dev(velInvMass), _dev(force_), dt,
                                             damping, n, int(fused_drift), _stream(stream)),
          "nbgb_integrate_reference_ex")


def measure_peak(which: str, iters: int = 4096, reps: int = 5):
    """Measured pipe throughput: 'ffma' / 'ffma2' / 'fadd2' / 'fmul2' /
    'ffma2_3op' (FLOP/s), 'mufu' (rsqrt/s), 'ex2' / 'lg2' (ops/s), or the
    register-resident pair interaction (20 FLOP/interaction) with 4 or 8
    source pairs per step: 'interact', 'interact_log1of4', 'interact_log2of4',
    'interact8', 'interact_log1of8' .. 'interact_log3of8' (that many source
    pairs in the log-domain form); 'dfma' (FP64 FLOP/s)."""
    code = {"ffma": 0, "ffma2": 1, "mufu": 2, "fadd2": 3, "fmul2": 4, "ffma2_3op": 5,
            "ffma2_mufu": 6, "ffma2_ffma": 7, "interact": 8, "ex2": 9, "lg2": 10,
            "interact_log1of4": 11, "interact_log2of4": 12, "interact8": 13,
            "interact_log1of8": 14, "interact_log2of8": 15, "interact_log3of8": 16,
            "dfma": 17}[which]
    rate, ms = ctypes.c_double(), ctypes.c_float()
    check(load().nbgb_measure_peak(code, iters, reps, ctypes.byref(rate), ctypes.byref(ms)),
          "nbgb_measure_peak")
    return rate.value, ms.value


def measure_copy(nbytes: int, reps: int = 21):
    """(GB/s, ms): one float4 copy kernel moving nbytes (half read, half
    written), L2 evicted before each launch, median of reps (CUDA events)."""
    gbs, ms = ctypes.c_double(), ctypes.c_float()
    check(load().nbgb_measure_copy(nbytes, reps, ctypes.byref(gbs), ctypes.byref(ms)),
          "nbgb_measure_copy")
    return gbs.value, ms.value


def last_status() -> int:
    return int(load().nbgb_last_status())


# ---------------------------------------------------------------------------
# Device-resident simulation
# ---------------------------------------------------------------------------
class System:
    """State resident in HBM; step() = force + integrate per step (reference
    integrators on the one-sided kernel: one launch, the integrate in the
    force kernel's epilogue; groups of 8 steps replay a CUDA graph), no host
    round trip."""

    def __init__(self, N: int, integrator: int = INTEGRATOR_REFERENCE,
                 softeningSquared: float = 1e-4, dt: float = 0.01, damping: float = 1.0):
        self.lib = load()
        self.n = N
        self.integrator = integrator
        self.h = self.lib.nbgb_system_create(N, integrator, softeningSquared, dt, damping)
        if not self.h:
            raise NbgbError(-6, "nbgb_system_create")

    def close(self):
        if self.h:
            self.lib.nbgb_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, posMass: np.ndarray, velInvMass: np.ndarray):
        pm = np.ascontiguousarray(posMass, np.float32)
        vm = np.ascontiguousarray(velInvMass, np.float32)
        assert pm.shape == (self.n, 4) and vm.shape == (self.n, 4)
        check(self.lib.nbgb_system_set_state(self.h, _f32p(pm), _f32p(vm)), "set_state")

    def set_state64(self, pos3: np.ndarray, vel3: np.ndarray, mass: np.ndarray):
        p = np.ascontiguousarray(pos3, np.float64)
        v = np.ascontiguousarray(vel3, np.float64)
        m = np.ascontiguousarray(mass, np.float32)
        check(self.lib.nbgb_system_set_state64(self.h, _f64p(p), _f64p(v), _f32p(m)),
              "set_state64")

    def step(self, nsteps: int = 1):
        check(self.lib.nbgb_system_step(self.h, nsteps), "step")

    def use_graph(self, enable: bool):
        check(self.lib.nbgb_system_set_graph(self.h, int(enable)), "set_graph")

    def set_force_algorithm(self, name: str):
        """'onesided' (default) or 'newton3'."""
        code = {"onesided": 0, "newton3": 1}[name]
        check(self.lib.nbgb_system_set_force_algorithm(self.h, code), "set_force_algorithm")

    def synchronize(self):
        check(self.lib.nbgb_system_synchronize(self.h), "synchronize")

    def sync_velocities(self):
        """KDK: apply the pending closing half kick now (the getters do it
        themselves)."""
        check(self.lib.nbgb_system_sync_velocities(self.h), "sync_velocities")

    def set_timing(self, enable: bool):
        check(self.lib.nbgb_system_set_timing(self.h, int(enable)), "set_timing")

    def last_force_ms(self) -> float:
        ms = ctypes.c_float()
        check(self.lib.nbgb_system_last_force_ms(self.h, ctypes.byref(ms)), "last_force_ms")
        return ms.value

    def last_integrate_ms(self):
        """(step_ms, half_kick_ms) of the latest timed integrate launches:
        the reference integrate or the FP64 kick+drift, and the closing FP64
        half kick (0.0 when none ran)."""
        a, b = ctypes.c_float(), ctypes.c_float()
        check(self.lib.nbgb_system_last_integrate_ms(self.h, ctypes.byref(a), ctypes.byref(b)),
              "last_integrate_ms")
        return a.value, b.value

    def get_state(self):
        pm = np.zeros((self.n, 4), np.float32)
        vm = np.zeros((self.n, 4), np.float32)
        check(self.lib.nbgb_system_get_state(self.h, _f32p(pm), _f32p(vm)), "get_state")
        return pm, vm

    def get_state64(self):
        p = np.zeros((self.n, 3), np.float64)
        v = np.zeros((self.n, 3), np.float64)
        check(self.lib.nbgb_system_get_state64(self.h, _f64p(p), _f64p(v)), "get_state64")
        return p, v

    def get_force(self) -> np.ndarray:
        f = np.zeros((self.n, 4), np.float32)
        check(self.lib.nbgb_system_get_force(self.h, _f32p(f)), "get_force")
        return f

    def diagnostics(self) -> dict:
        """FP64 kinetic/potential/total energy, momentum, angular momentum."""
        out = np.zeros(8, np.float64)
        check(self.lib.nbgb_system_diagnostics(self.h, _f64p(out)), "diagnostics")
        return {"kinetic": out[0], "potential": out[1], "energy": out[0] + out[1],
                "momentum": out[2:5].copy(), "angular_momentum": out[5:8].copy()}

    def set_plan(self, config: int = -1, nsplit: int = -1):
        """Force the one-sided kernel's plan (as for force(); -1, -1: the
        planner's choice)."""
        check(self.lib.nbgb_system_set_plan(self.h, config, nsplit), "set_plan")

    def plan(self):
        c, s = ctypes.c_int(), ctypes.c_int()
        check(self.lib.nbgb_system_plan(self.h, ctypes.byref(c), ctypes.byref(s)), "plan")
        return c.value, s.value

    @property
    def stream(self) -> int:
        return int(self.lib.nbgb_system_stream(self.h) or 0)


class Ensemble:
    """Many independent systems resident in one device arena; tick() moves
    all of them one FP64 KDK step with one persistent force launch."""

    def __init__(self, max_bodies: int, max_systems: int, softeningSquared: float = 1e-4,
                 tuning="auto"):
        """tuning: "auto" applies the autotuner's table (nbody_gb300/tuning/
        ensemble.json) when present, a dict applies that table, None keeps the
        library's default per-bucket rule."""
        self.lib = load()
        self.h = self.lib.nbgb_ensemble_create(max_bodies, max_systems, softeningSquared)
        if not self.h:
            raise NbgbError(-6, "nbgb_ensemble_create")
        self._n = {}
        if tuning is not None:
            from . import autotune
            autotune.apply(self, autotune.load() if tuning == "auto" else tuning)

    def close(self):
        if self.h:
            self.lib.nbgb_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def device_bytes(self) -> int:
        return int(self.lib.nbgb_ensemble_device_bytes(self.h))

    def set_bucket_plan(self, bucket: int, variant: int, jt: int = 256, nsplit: int = 1):
        check(self.lib.nbgb_ensemble_set_bucket_plan(self.h, bucket, variant, jt, nsplit),
              "set_bucket_plan")

    def add(self, pos3, vel3, mass, dt: float, steps: int):
        """Admit a system; returns its slot, or None when the arena is full."""
        p = np.ascontiguousarray(pos3, np.float64)
        v = np.ascontiguousarray(vel3, np.float64)
        m = np.ascontiguousarray(mass, np.float32)
        slot = ctypes.c_int(-1)
        rc = self.lib.nbgb_ensemble_add(self.h, _f64p(p), _f64p(v), _f32p(m), p.shape[0], dt,
                                        steps, ctypes.byref(slot))
        if rc == -6:
            return None
        check(rc, "ensemble_add")
        self._n[slot.value] = p.shape[0]
        return slot.value

    def tick(self, n: int = 1):
        check(self.lib.nbgb_ensemble_tick(self.h, n), "ensemble_tick")

    def use_graph(self, enable: bool):
        check(self.lib.nbgb_ensemble_set_graph(self.h, int(enable)), "ensemble_set_graph")

    def synchronize(self):
        check(self.lib.nbgb_ensemble_synchronize(self.h), "ensemble_synchronize")

    def finished(self, max_n: int = 65536):
        buf = (ctypes.c_int * max_n)()
        k = self.lib.nbgb_ensemble_finished(self.h, buf, max_n)
        if k < 0:
            check(k, "ensemble_finished")
        return [buf[i] for i in range(k)]

    def get_state(self, slot: int):
        n = self._n[slot]
        p = np.zeros((n, 3), np.float64)
        v = np.zeros((n, 3), np.float64)
        a = np.zeros((n, 4), np.float32)
        check(self.lib.nbgb_ensemble_get_state(self.h, slot, _f64p(p), _f64p(v), _f32p(a)),
              "ensemble_get_state")
        return p, v, a

    def slot_info(self, slot: int) -> dict:
        info = np.zeros(6, np.int64)
        check(self.lib.nbgb_ensemble_slot_info(
            self.h, slot, info.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))), "slot_info")
        return {"n": int(info[0]), "steps_done": int(info[1]), "steps_left": int(info[2]),
                "variant": int(info[3]), "jt": int(info[4]), "nsplit": int(info[5])}

    def set_substeps(self, slot: int, sub: int):
        """Steps this system takes per tick (1..8) from the next tick on; it
        then finishes after 1 + ceil(steps / sub) ticks."""
        check(self.lib.nbgb_ensemble_set_substeps(self.h, slot, sub), "ensemble_set_substeps")

    def set_grid(self, ctas: int):
        """CTAs of the persistent force launch (0 = all resident slots)."""
        check(self.lib.nbgb_ensemble_set_grid(self.h, ctas), "ensemble_set_grid")

    def max_grid(self) -> int:
        return int(self.lib.nbgb_ensemble_max_grid(self.h))

    def set_priority(self, high: bool):
        """High: the ensemble's stream gets the device's greatest priority."""
        check(self.lib.nbgb_ensemble_set_priority(self.h, int(high)), "ensemble_set_priority")

    def set_newton3_min(self, nmin: int):
        """Systems admitted afterwards with N >= nmin use the Newton's-third-
        law kernel (0 = none); results then repeat to FP64 rounding order."""
        check(self.lib.nbgb_ensemble_set_newton3_min(self.h, nmin), "ensemble_set_newton3_min")

    def remove(self, slot: int):
        check(self.lib.nbgb_ensemble_remove(self.h, slot), "ensemble_remove")
        self._n.pop(slot, None)

    def active(self) -> int:
        return int(self.lib.nbgb_ensemble_active(self.h))


# ---------------------------------------------------------------------------
# Initial conditions, metrics (host)
# ---------------------------------------------------------------------------
def ic_reference(N: int, seed: int = REFERENCE_SEED, scale: float = REFERENCE_SCALE,
                 velscale: float = REFERENCE_VELOCITY_SCALE):
    """The reference driver's bodies (src/nbody_util.cpp:102-144)."""
    pm = np.zeros((N, 4), np.float32)
    vm = np.zeros((N, 4), np.float32)
    check(load().nbgb_ic_reference(_f32p(pm), _f32p(vm), N, scale, velscale, seed),
          "ic_reference")
    return pm, vm


def ic_uniform_ball(N: int, seed: int, radius: float = 1.0, m_lo: float = 1.0,
                    m_hi: float = 1.0):
    """Uniform ball; mass U[m_lo, m_hi]/N (equal 1/N by default); v = 0."""
    pm = np.zeros((N, 4), np.float32)
    vm = np.zeros((N, 4), np.float32)
    check(load().nbgb_ic_uniform_ball(_f32p(pm), _f32p(vm), N, radius, m_lo, m_hi, seed),
          "ic_uniform_ball")
    return pm, vm


def ic_plummer(N: int, seed: int):
    """Plummer sphere (G=M=a=1): (pos3 f64, vel3 f64, posMass f32, velInvMass f32)."""
    p = np.zeros((N, 3), np.float64)
    v = np.zeros((N, 3), np.float64)
    pm = np.zeros((N, 4), np.float32)
    vm = np.zeros((N, 4), np.float32)
    check(load().nbgb_ic_plummer(_f64p(p), _f64p(v), _f32p(pm), _f32p(vm), N, seed),
          "ic_plummer")
    return p, v, pm, vm


def force_f64_host(posMass: np.ndarray, softeningSquared: float, idx) -> tuple:
    """FP64 force (n,3) and potential (n,) of targets idx (host threads)."""
    pm = np.ascontiguousarray(posMass, np.float32)
    idx = np.ascontiguousarray(idx, np.int64)
    f = np.zeros((idx.shape[0], 3), np.float64)
    phi = np.zeros(idx.shape[0], np.float64)
    check(load().nbgb_force_f64_host(_f32p(pm), pm.shape[0], float(np.float32(softeningSquared)),
                                     idx.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                     idx.shape[0], _f64p(f), _f64p(phi)), "force_f64_host")
    return f, phi


def crosscheck_max_rel_error(force_: np.ndarray, golden: np.ndarray) -> float:
    f = np.ascontiguousarray(force_, np.float32)
    g = np.ascontiguousarray(golden, np.float32)
    return float(load().nbgb_crosscheck_max_rel_error(_f32p(f), _f32p(g), f.shape[0]))


def force_error_stats(force_: np.ndarray, truth3: np.ndarray, idx=None):
    """(max, rms) of per-body |F - T| / |T| against FP64 truth rows."""
    f = np.ascontiguousarray(force_, np.float32)
    t = np.ascontiguousarray(truth3, np.float64)
    mx, rms = ctypes.c_double(), ctypes.c_double()
    ip = None
    if idx is not None:
        idx = np.ascontiguousarray(idx, np.int64)
        ip = idx.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))
    check(load().nbgb_force_error_stats(_f32p(f), _f64p(t), ip, t.shape[0], ctypes.byref(mx),
                                        ctypes.byref(rms)), "force_error_stats")
    return mx.value, rms.value


def bucket_of(n: int) -> int:
    """Ensemble plan bucket of a system size: N in [2^b, 2^(b+1))."""
    return max(0, int(n).bit_length() - 1)


def interactions_per_second(N: int, ms: float) -> float:
    """src/nbody.cu:1026: N^2 interactions (self pairs included) per ms."""
    return float(N) * float(N) * 1000.0 / ms


def reference_line(name: str, N: int, ms: float, rel_error=None, name_width: int = 0) -> str:
    """The reference's per-step stdout line (src/nbody.cu:1024-1053)."""
    ips = interactions_per_second(N, ms)
    gflops = ips * FLOPS_PER_INTERACTION * 1e-9
    if ips > 1e9:
        s = f"{name:>{name_width}}: {ms:8.2f} ms = {ips / 1e9:8.3f}x10^9 interactions/s ({gflops:9.2f} GFLOPS)"
    else:
        s = f"{name:>{name_width}}: {ms:8.2f} ms = {ips / 1e6:8.3f}x10^6 interactions/s ({gflops:9.2f} GFLOPS)"
    if rel_error is not None:
        s += f" (Rel. error: {rel_error:E})"
    return s
