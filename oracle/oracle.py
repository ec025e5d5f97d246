"""ctypes front end of the CPU checker (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module.  It loads the C restatement built by oracle/Makefile and, when
present, the reference's own CPU objects (oracle/_ref/libnbody_ref.so).

Function map (reference file:line each one follows):
  forces_aos        src/nbody_CPU_AOS.cpp:51-98   (C restatement)
  forces_soa        src/nbody_CPU_SOA.cpp:53-105  (C restatement, bounded i-range)
  forces_f64        FP64 all-pairs sum, no reference counterpart
  integrate         src/nbody.cu:158-236          (integrateOne per body)
  max_rel_error     src/nbody.cu:120-125, 406-418 (crosscheck metric)
  random_unit_bodies src/nbody_util.cpp:81-144    (LCG initial conditions)
  forces_aos_idx    src/nbody_CPU_AOS.cpp:60-95   (CPU_AOS for listed targets)
  integrate_contracted  src/nbody.cu:158-236 as the reference's own build
                    compiles it (position update fused)
  ic_plummer        the GB300 library's Plummer generator, restated (inputs
                    for the CPU baseline without loading that library)
  ref().forces_aos / forces_soa / random_unit_bodies: the reference's own
                    compiled objects (ComputeGravitation_AOS/_SOA,
                    randomUnitBodies), only where oracle/_ref was built;
  ref_driver().integrate: the reference driver's integrateGravitation_SOA
                    (oracle/ref_shim.cpp), likewise.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_REF = os.path.join(_HERE, "_ref")

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_longlong)


def reference_dir() -> str | None:
    """The reference checkout named by NBODY_REF_DIR, when it has its sources
    (no default: machines without the reference build the restatement only)."""
    d = os.environ.get("NBODY_REF_DIR")
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def build(ref: bool = False) -> None:
    """Compile the restatement (and, if asked and present, the reference)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    d = reference_dir()
    if ref and d:
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={d}"], check=True)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class _Orc:
    def __init__(self, path: str):
        lib = ctypes.CDLL(path)
        lib.orc_forces_aos.argtypes = [_f32p, _f32p, ctypes.c_float, ctypes.c_size_t]
        lib.orc_forces_soa.argtypes = [_f32p] * 7 + [ctypes.c_float, ctypes.c_size_t,
                                                     ctypes.c_size_t, ctypes.c_size_t]
        lib.orc_forces_f64.argtypes = [_f64p, _f32p, ctypes.c_double, ctypes.c_size_t,
                                       _i64p, ctypes.c_size_t]
        lib.orc_potential_f64.argtypes = [_f64p, _f32p, ctypes.c_double, ctypes.c_size_t,
                                          _i64p, ctypes.c_size_t]
        lib.orc_integrate.argtypes = [_f32p, _f32p, _f32p, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_size_t]
        lib.orc_max_rel_error.argtypes = [_f32p, _f32p, ctypes.c_size_t]
        lib.orc_max_rel_error.restype = ctypes.c_float
        lib.orc_random_unit_bodies.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_float,
                                               ctypes.c_float, ctypes.c_uint32]
        lib.orc_num_threads.restype = ctypes.c_int
        lib.orc_forces_aos_idx.argtypes = [_f32p, _f32p, ctypes.c_float, ctypes.c_size_t,
                                           _i64p, ctypes.c_size_t]
        lib.orc_integrate_contracted.argtypes = lib.orc_integrate.argtypes
        lib.orc_ic_plummer.argtypes = [_f64p, _f64p, _f32p, ctypes.c_size_t, ctypes.c_uint64]
        self.lib = lib

    def forces_aos(self, posMass: np.ndarray, eps2: float) -> np.ndarray:
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        out = np.zeros_like(pm)
        self.lib.orc_forces_aos(_ptr(out, _f32p), _ptr(pm, _f32p), eps2, pm.shape[0])
        return out

    def forces_aos_idx(self, posMass: np.ndarray, eps2: float, idx) -> np.ndarray:
        """CPU_AOS sums for the listed target bodies only: (len(idx), 4)."""
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        assert idx.size == 0 or (idx.min() >= 0 and idx.max() < pm.shape[0])
        out = np.zeros((idx.shape[0], 4), np.float32)
        self.lib.orc_forces_aos_idx(_ptr(out, _f32p), _ptr(pm, _f32p), eps2, pm.shape[0],
                                    _ptr(idx, _i64p), idx.shape[0])
        return out

    def forces_soa(self, posMass: np.ndarray, eps2: float, i_begin: int = 0,
                   i_end: int | None = None) -> np.ndarray:
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        n = pm.shape[0]
        i_end = n if i_end is None else i_end
        p = [np.ascontiguousarray(pm[:, c]) for c in range(4)]
        f = [np.zeros(n, np.float32) for _ in range(3)]
        self.lib.orc_forces_soa(*(_ptr(a, _f32p) for a in f), *(_ptr(a, _f32p) for a in p),
                                eps2, n, i_begin, i_end)
        out = np.zeros((n, 4), np.float32)
        for c in range(3):
            out[:, c] = f[c]
        return out

    def soa_timer(self, posMass: np.ndarray, eps2: float):
        """Return a zero-argument callable running the SOA loop over a fixed
        i-range, with all array conversion done up front (for timing)."""
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        n = pm.shape[0]
        p = [np.ascontiguousarray(pm[:, c]) for c in range(4)]
        f = [np.zeros(n, np.float32) for _ in range(3)]
        args_fixed = [_ptr(a, _f32p) for a in f] + [_ptr(a, _f32p) for a in p]

        def run(i_begin: int, i_end: int):
            self.lib.orc_forces_soa(*args_fixed, eps2, n, i_begin, i_end)
            return f
        return run

    def forces_f64(self, posMass: np.ndarray, eps2: float, idx=None) -> np.ndarray:
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        if idx is None:
            nt = pm.shape[0]
            ip = None
        else:
            idx = np.ascontiguousarray(idx, dtype=np.int64)
            nt = idx.shape[0]
            ip = _ptr(idx, _i64p)
        out = np.zeros((nt, 3), np.float64)
        self.lib.orc_forces_f64(_ptr(out, _f64p), _ptr(pm, _f32p), eps2, pm.shape[0], ip, nt)
        return out

    def potential_f64(self, posMass: np.ndarray, eps2: float, idx=None) -> np.ndarray:
        pm = np.ascontiguousarray(posMass, dtype=np.float32).reshape(-1, 4)
        if idx is None:
            nt, ip = pm.shape[0], None
        else:
            idx = np.ascontiguousarray(idx, dtype=np.int64)
            nt, ip = idx.shape[0], _ptr(idx, _i64p)
        out = np.zeros(nt, np.float64)
        self.lib.orc_potential_f64(_ptr(out, _f64p), _ptr(pm, _f32p), eps2, pm.shape[0], ip, nt)
        return out

    def integrate(self, posMass, velInvMass, force, dt: float, damping: float):
        """In place on float32 (N,4) arrays, like the reference."""
        for a in (posMass, velInvMass, force):
            assert a.dtype == np.float32 and a.flags.c_contiguous
        self.lib.orc_integrate(_ptr(posMass, _f32p), _ptr(velInvMass, _f32p),
                               _ptr(force, _f32p), dt, damping, posMass.shape[0])

    def integrate_contracted(self, posMass, velInvMass, force, dt: float, damping: float):
        """As integrate, with the position update fused (fmaf), the way the
        reference's own build (-O3 -ffast-math -march=native) compiles it."""
        for a in (posMass, velInvMass, force):
            assert a.dtype == np.float32 and a.flags.c_contiguous
        self.lib.orc_integrate_contracted(_ptr(posMass, _f32p), _ptr(velInvMass, _f32p),
                                          _ptr(force, _f32p), dt, damping, posMass.shape[0])

    def ic_plummer(self, n: int, seed: int):
        """Plummer sphere as the GB300 library's nbgb_ic_plummer makes it:
        (pos3 float64 (n,3), vel3 float64 (n,3), posMass float32 (n,4))."""
        p = np.zeros((n, 3), np.float64)
        v = np.zeros((n, 3), np.float64)
        pm = np.zeros((n, 4), np.float32)
        self.lib.orc_ic_plummer(_ptr(p, _f64p), _ptr(v, _f64p), _ptr(pm, _f32p), n,
                                seed % (1 << 64))
        return p, v, pm

    def max_rel_error(self, force, golden) -> float:
        f = np.ascontiguousarray(force, dtype=np.float32)
        g = np.ascontiguousarray(golden, dtype=np.float32)
        return float(self.lib.orc_max_rel_error(_ptr(f, _f32p), _ptr(g, _f32p), f.shape[0]))

    def random_unit_bodies(self, n: int, seed: int, scale: float = 0.9, velscale: float = 8.0):
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        self.lib.orc_random_unit_bodies(_ptr(pos, _f32p), _ptr(vel, _f32p), n, scale,
                                        velscale, seed)
        return pos, vel

    def num_threads(self) -> int:
        return int(self.lib.orc_num_threads())


_cache: dict[str, object] = {}


def fast_flags() -> str:
    """The compiler flags of liborc_fast.so on this machine (oracle/Makefile)."""
    import platform
    extra = " -mlow-precision-recip-sqrt -mtune=native" if platform.machine() == "aarch64" else ""
    return "gcc -O3 -ffast-math -fopenmp -march=native" + extra


def ieee() -> _Orc:
    """Restatement with IEEE binary32 semantics (deterministic j order)."""
    if "ieee" not in _cache:
        _cache["ieee"] = _Orc(os.path.join(_BUILD, "liborc_ieee.so"))
    return _cache["ieee"]


def fast() -> _Orc:
    """Restatement compiled with the reference's CPU flags (timed baseline)."""
    if "fast" not in _cache:
        _cache["fast"] = _Orc(os.path.join(_BUILD, "liborc_fast.so"))
    return _cache["fast"]


class _Ref:
    """The reference's own CPU objects (ComputeGravitation_AOS / _SOA)."""

    def __init__(self, path: str):
        lib = ctypes.CDLL(path)
        lib.ComputeGravitation_AOS.argtypes = [_f32p, _f32p, ctypes.c_float, ctypes.c_size_t]
        lib.ComputeGravitation_AOS.restype = ctypes.c_float
        lib.ComputeGravitation_SOA.argtypes = [ctypes.POINTER(_f32p), ctypes.POINTER(_f32p),
                                               _f32p, ctypes.c_float, ctypes.c_size_t]
        lib.ComputeGravitation_SOA.restype = ctypes.c_float
        lib.seedRandom.argtypes = [ctypes.c_uint]
        lib.randomUnitBodies.argtypes = [_f32p, _f32p, ctypes.c_size_t, ctypes.c_float,
                                         ctypes.c_float]
        self.lib = lib

    @staticmethod
    def _aligned(shape, dtype=np.float32):
        # The reference asserts 64-byte alignment (src/nbody_util.h:45).
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        raw = np.zeros(nbytes + 64, np.uint8)
        off = (-raw.ctypes.data) % 64
        return raw[off:off + nbytes].view(dtype).reshape(shape)

    def forces_aos(self, posMass: np.ndarray, eps2: float) -> np.ndarray:
        n = posMass.shape[0]
        assert n % 1024 == 0 and n >= 1024, "the reference requires N % 1024 == 0"
        pm = self._aligned((n, 4))
        pm[:] = posMass
        out = self._aligned((n, 4))
        self.lib.ComputeGravitation_AOS(_ptr(out, _f32p), _ptr(pm, _f32p), eps2, n)
        return np.array(out)

    def forces_soa(self, posMass: np.ndarray, eps2: float) -> np.ndarray:
        n = posMass.shape[0]
        assert n % 1024 == 0 and n >= 1024, "the reference requires N % 1024 == 0"
        pos = [self._aligned((n,)) for _ in range(3)]
        frc = [self._aligned((n,)) for _ in range(3)]
        mass = self._aligned((n,))
        for c in range(3):
            pos[c][:] = posMass[:, c]
        mass[:] = posMass[:, 3]
        pp = (_f32p * 3)(*[_ptr(a, _f32p) for a in pos])
        fp = (_f32p * 3)(*[_ptr(a, _f32p) for a in frc])
        self.lib.ComputeGravitation_SOA(fp, pp, _ptr(mass, _f32p), eps2, n)
        out = np.zeros((n, 4), np.float32)
        for c in range(3):
            out[:, c] = frc[c]
        return out

    def random_unit_bodies(self, n: int, seed: int, scale: float = 0.9, velscale: float = 8.0):
        pos = self._aligned((n, 4))
        vel = self._aligned((n, 4))
        self.lib.seedRandom(seed)
        self.lib.randomUnitBodies(_ptr(pos, _f32p), _ptr(vel, _f32p), n, scale, velscale)
        return np.array(pos), np.array(vel)


def ref_available() -> bool:
    return os.path.exists(os.path.join(_REF, "libnbody_ref.so"))


class _RefDriver:
    """The reference driver's own integrator, integrateGravitation_SOA
    (src/nbody.cu:186-236), exported by oracle/ref_shim.cpp."""

    def __init__(self, path: str):
        lib = ctypes.CDLL(path)
        lib.ref_integrate_soa.argtypes = [_f32p] * 10 + [ctypes.c_float, ctypes.c_float,
                                                          ctypes.c_size_t]
        self.lib = lib

    def integrate(self, posMass, velInvMass, force, dt: float, damping: float):
        """In place on float32 (N,4) arrays (N % 1024 == 0, as the reference
        requires), through the reference's SOA arrays."""
        n = posMass.shape[0]
        assert n % 1024 == 0 and n >= 1024, "the reference requires N % 1024 == 0"
        cols = {}
        for name, a in (("p", posMass), ("v", velInvMass), ("f", force)):
            for c in range(4 if name != "f" else 3):
                b = _Ref._aligned((n,))
                b[:] = a[:, c]
                cols[name, c] = b
        args = [cols["p", 0], cols["p", 1], cols["p", 2], cols["v", 3], cols["v", 0],
                cols["v", 1], cols["v", 2], cols["f", 0], cols["f", 1], cols["f", 2]]
        self.lib.ref_integrate_soa(*(_ptr(a, _f32p) for a in args), dt, damping, n)
        for c in range(3):
            posMass[:, c] = cols["p", c]
            velInvMass[:, c] = cols["v", c]


def ref_driver_available() -> bool:
    return os.path.exists(os.path.join(_REF, "libnbody_refdrv.so"))


def ref_driver() -> _RefDriver:
    if "refdrv" not in _cache:
        _cache["refdrv"] = _RefDriver(os.path.join(_REF, "libnbody_refdrv.so"))
    return _cache["refdrv"]


def ref() -> _Ref:
    if "ref" not in _cache:
        _cache["ref"] = _Ref(os.path.join(_REF, "libnbody_ref.so"))
    return _cache["ref"]


# --------------------------------------------------------------------------
# Error statistics used by every parity test.
# --------------------------------------------------------------------------
def per_body_rel_error(force: np.ndarray, truth: np.ndarray):
    """max and RMS over bodies of |F - T| / |T| (xyz only)."""
    f = np.asarray(force, np.float64)[:, :3]
    t = np.asarray(truth, np.float64)[:, :3]
    num = np.linalg.norm(f - t, axis=1)
    den = np.linalg.norm(t, axis=1)
    rel = num / np.where(den > 0, den, 1.0)
    return float(rel.max()), float(np.sqrt(np.mean(rel * rel)))
