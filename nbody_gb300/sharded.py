"""Row-sharded force evaluation and step loop: one process per GPU.

The reference's multi-GPU algorithm (ComputeGravitation_multiGPU,
src/nbody_multiGPU.cu:65-140) runs single-threaded over all GPUs: it copies
the whole posMass array to every GPU, each GPU evaluates the forces on its
N/G target rows against all N sources (ComputeNBodyGravitation_multiGPU,
src/nbody_multiGPU.cu:47-63), and the force slices are copied back into one
host array.  Here one process drives one GPU (torch.distributed; NCCL between
GPUs) and the exchange stays on the devices:

  row split       rank r owns rows [r R, min(N, (r+1) R)), R = ceil(N / world)
                  (any N; the reference requires N % GPUs == 0)
  sharded_force   every rank holds all N posMass; nbgb_force_rows evaluates
                  its rows against all N sources into its slice of a padded
                  (world x R) force array, and one all-gather of the slices
                  gives every rank the whole force array, as the reference's
                  host array holds it
  ShardedSystem   state resident on the devices; a step is the rank's force
                  rows, the reference integrator on its own rows (in place on
                  its slice of posMass and its velocities), then one
                  all-gather of the posMass slices (16 B x R per rank), which
                  gives every rank the sources of the next force pass: the
                  only exchange per step

The force kernel's bulk copies read only the rank's own HBM: the all-gather
lands in a local buffer first (no peer or multicast loads).  Rank-local
compute goes through the library; `force_rows_fn` / `integrate_fn` exist so
the partitioning and exchange can be exercised without a GPU (the library
itself has no CPU path).
"""
from __future__ import annotations

import numpy as np


def row_range(n: int, world: int, rank: int):
    """(begin, end, R) of rank's rows: R = ceil(n / world) rows per rank,
    the last ranks possibly shorter or empty."""
    r = -(-n // world) if n else 0
    return min(n, rank * r), min(n, (rank + 1) * r), r


def _all_gather_rows(store, seg, group=None):
    """store: (world * R, 4) tensor; seg: this rank's (R, 4) segment of it.
    Afterwards every segment of store holds its owner's rows."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    if world == 1:
        return
    if dist.get_backend(group) == "nccl":
        dist.all_gather_into_tensor(store, seg.clone(), group=group)
    else:
        parts = list(store.split(seg.shape[0]))
        dist.all_gather(parts, seg.clone(), group=group)


def _default_force_rows(pm, eps2, r0, r1, out):
    from . import force_rows
    force_rows(pm, eps2, r0, r1, out=out)


def _default_integrate(pm_rows, vel_rows, force_rows_, dt, damping, fused_drift):
    from . import integrate_reference
    integrate_reference(pm_rows, vel_rows, force_rows_, dt, damping, fused_drift=fused_drift)


def sharded_force(posMass, softeningSquared: float, group=None, force_rows_fn=None):
    """The multi-GPU algorithm row: posMass (N,4) holds all bodies on every
    rank; returns the (N,4) forces, identical on every rank."""
    import torch
    import torch.distributed as dist
    n = posMass.shape[0]
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    r0, r1, r = row_range(n, world, rank)
    store = torch.zeros((world * r, 4), dtype=torch.float32, device=posMass.device)
    seg = store[rank * r:(rank + 1) * r]
    if r1 > r0:
        (force_rows_fn or _default_force_rows)(posMass, softeningSquared, r0, r1,
                                               seg[:r1 - r0])
    _all_gather_rows(store, seg, group)
    return store[:n]


class ShardedSystem:
    """N bodies stepped by `world` ranks with the reference integrator
    (integrateOne, src/nbody.cu:158-182; fused_drift as the reference binary
    computes it).  Every rank keeps all N posMass (the next force pass's
    sources) and the velocities of its own rows."""

    def __init__(self, n: int, softeningSquared: float = 1e-4, dt: float = 0.01,
                 damping: float = 1.0, device=None, group=None, fused_drift: bool = False,
                 force_rows_fn=None, integrate_fn=None):
        import torch
        import torch.distributed as dist
        self.n, self.eps2, self.dt, self.damping = n, softeningSquared, dt, damping
        self.group = group
        self.world, self.rank = dist.get_world_size(group), dist.get_rank(group)
        self.r0, self.r1, self.R = row_range(n, self.world, self.rank)
        self.fused_drift = fused_drift
        dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
        self.store = torch.zeros((self.world * self.R, 4), dtype=torch.float32, device=dev)
        self.seg = self.store[self.rank * self.R:(self.rank + 1) * self.R]
        self.vel = torch.zeros((self.R, 4), dtype=torch.float32, device=dev)
        self.force = torch.zeros((self.R, 4), dtype=torch.float32, device=dev)
        self.force_rows_fn = force_rows_fn or _default_force_rows
        self.integrate_fn = integrate_fn or _default_integrate

    @property
    def rows(self) -> int:
        return self.r1 - self.r0

    def set_state(self, posMass: np.ndarray, velInvMass: np.ndarray):
        """Host (N,4) arrays, the same on every rank."""
        import torch
        assert posMass.shape == (self.n, 4) and velInvMass.shape == (self.n, 4)
        self.store[:self.n] = torch.from_numpy(np.ascontiguousarray(posMass, np.float32))
        self.vel[:self.rows] = torch.from_numpy(
            np.ascontiguousarray(velInvMass[self.r0:self.r1], np.float32))

    def step(self, nsteps: int = 1):
        pm = self.store[:self.n]
        k = self.rows
        for _ in range(nsteps):
            if k:
                self.force_rows_fn(pm, self.eps2, self.r0, self.r1, self.force[:k])
                self.integrate_fn(self.seg[:k], self.vel[:k], self.force[:k], self.dt,
                                  self.damping, self.fused_drift)
            _all_gather_rows(self.store, self.seg, self.group)

    def get_state(self):
        """(posMass, velInvMass) of all N bodies as host arrays (collective:
        every rank must call it)."""
        import torch
        vstore = torch.zeros_like(self.store)
        vseg = vstore[self.rank * self.R:(self.rank + 1) * self.R]
        vseg[:self.rows] = self.vel[:self.rows]
        _all_gather_rows(vstore, vseg, self.group)
        return self.store[:self.n].cpu().numpy(), vstore[:self.n].cpu().numpy()

    def get_force(self) -> np.ndarray:
        """This rank's force rows of the latest step (host array)."""
        return self.force[:self.rows].cpu().numpy()
