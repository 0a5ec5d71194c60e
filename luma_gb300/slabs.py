"""Decomposition of a level-0 grid into slabs along x, one per GPU.

The counterpart of the reference's MPI decomposition: MpiManager builds a
Cartesian topology of sub-domains with a halo around each
(src/MpiManager.cpp:228-560) and after every step of a grid exchanges the
populations of the layers along each cut with the neighbours
(MpiManager::mpi_communicate, :631-820, packing with mpi_buffer_pack and
unpacking with mpi_buffer_unpack, src/Mpi_buffer_pack.cpp,
src/Mpi_buffer_unpk.cpp; called at the end of GridObj::LBM_multi_opt,
src/GridObj_ops_lbm_optimised.cpp:189).

Here each slab is an ordinary grid (luma_gpu_grid, or an oracle grid on the
host) holding its real x-planes plus one ghost plane on each side; it steps
with the unchanged kernels, and after every step it hands its first and
last real planes to its neighbours, which put them in their ghost planes
(luma_gpu_planes_export / luma_gpu_planes_import: every population of the
plane, as the reference packs every population of a halo site).  The ghost
planes' own updates are never read: the exchange overwrites them before the
next step pulls from them.  So the real sites of the slabs see exactly the
arithmetic of the undivided grid.

Transports: ``LocalExchange`` for slabs held by one process (on one GPU,
device buffers); ``DistExchange`` for one slab per rank over
torch.distributed point-to-point send/receive (NCCL with device buffers on
GPUs, gloo with host buffers), each rank sending to and receiving from its
two neighbours on a ring.  No collective is involved.

Scope: grids periodic along x whose sites are fluid, solid or slip (their
stream reads nothing of a neighbour but populations); no sub-grids, IB or
BFL bodies, velocity or pressure boundaries across a cut.  The slabs are
created with LUMA_FLAG_TWO_BUFFER (the in-place step alternates storage
layouts, which a plane copy does not follow).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import _abi as A

ALLOWED_SITES = (A.FLUID, A.SOLID, A.SLIP)


def partition(n: int, nslabs: int) -> list[tuple[int, int]]:
    """[start, end) x-plane ranges of nslabs slabs over n planes, the first
    n % nslabs slabs one plane wider."""
    if nslabs <= 0 or nslabs > n:
        raise ValueError(f"cannot cut {n} planes into {nslabs} slabs")
    base, extra = divmod(n, nslabs)
    out, a = [], 0
    for r in range(nslabs):
        b = a + base + (1 if r < extra else 0)
        out.append((a, b))
        a = b
    return out


def ghost_planes(n: int, start: int, end: int) -> np.ndarray:
    """Global x-planes of a slab's local planes: the left ghost, the real
    planes start..end-1, the right ghost (periodic along x)."""
    return np.array([(start - 1) % n, *range(start, end), end % n])


def slab_level(l0, start: int, end: int):
    """The slab [start, end) of a level-0 grid as a level-0 grid of its own
    (labels, positions, state of its local planes; the global edges stay)."""
    d = l0.defs
    typ = np.asarray(l0.typ).reshape(l0.N, l0.M, l0.K)
    bad = ~np.isin(typ, ALLOWED_SITES)
    if bad.any():
        raise ValueError("slabs take fluid, solid and slip sites only (a boundary condition across a cut reads "
                         "more of its neighbour than its populations)")
    planes = ghost_planes(l0.N, start, end)
    D = d.dims

    def cut(a, per_site):
        if a is None:
            return None
        return np.ascontiguousarray(np.asarray(a).reshape(l0.N, l0.M, l0.K, per_site)[planes]).reshape(-1)

    return dataclasses.replace(
        l0, N=len(planes), typ=cut(l0.typ, 1).astype(np.int32), xpos=np.ascontiguousarray(np.asarray(l0.xpos)[planes]),
        u=cut(l0.u, D), rho=cut(l0.rho, 1), force_xyz=cut(l0.force_xyz, D))


class GpuSlab:
    """A slab on a GPU: a GpuGrid whose halo planes move through device
    buffers (torch tensors)."""

    def __init__(self, level, precision: int, device=None, flags: int = 0):
        import torch
        from .gpu import GpuGrid
        desc = level.desc(precision=precision)
        desc.flags |= A.FLAG_TWO_BUFFER | flags
        self.level = level
        self.grid = GpuGrid(desc)
        self.n_local = level.N
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        nb = self.grid.planes_bytes(1)
        self.send = [torch.empty(nb, dtype=torch.uint8, device=self.device) for _ in range(2)]
        self.recv = [torch.empty(nb, dtype=torch.uint8, device=self.device) for _ in range(2)]

    def upload(self, f, u, rho, force=None, t=0):
        self.grid.upload(f, u, rho, force, t)

    def step(self, n: int = 1):
        self.grid.step(n)

    def pack(self):
        """First and last real planes into the send buffers (left, right)."""
        self.grid.planes_export(1, 1, self.send[0].data_ptr())
        self.grid.planes_export(self.n_local - 2, 1, self.send[1].data_ptr())

    def unpack(self):
        """The receive buffers (from the left, from the right) into the ghost planes."""
        self.grid.planes_import(0, 1, self.recv[0].data_ptr())
        self.grid.planes_import(self.n_local - 1, 1, self.recv[1].data_ptr())

    def synchronize(self):
        self.grid.synchronize()

    def download(self):
        return self.grid.download()

    def close(self):
        self.grid.close()


class HostSlab:
    """A slab held by a host grid with the oracle's interface (upload /
    step / download in the reference's layout): halo planes as float64
    tensors of the plane's populations in the reference's site order.
    Used for the exchange logic on CPU ranks."""

    def __init__(self, level, grid):
        import torch
        self.level = level
        self.grid = grid
        self.n_local = level.N
        self.Q = level.defs.Q
        self.site_vals = level.M * level.K * self.Q
        self.send = [torch.empty(self.site_vals, dtype=torch.float64) for _ in range(2)]
        self.recv = [torch.empty(self.site_vals, dtype=torch.float64) for _ in range(2)]

    def upload(self, f, u, rho, force=None, t=0):
        self.grid.upload(f, u, rho, force, t)

    def step(self, n: int = 1):
        self.grid.step(n)

    def _plane(self, f, i):
        return f[i * self.site_vals:(i + 1) * self.site_vals]

    def pack(self):
        import torch
        f = self.grid.download()["f"]
        self.send[0].copy_(torch.from_numpy(self._plane(f, 1).copy()))
        self.send[1].copy_(torch.from_numpy(self._plane(f, self.n_local - 2).copy()))

    def unpack(self):
        st = self.grid.download()
        f = st["f"]
        self._plane(f, 0)[:] = self.recv[0].numpy()
        self._plane(f, self.n_local - 1)[:] = self.recv[1].numpy()
        self.grid.upload(f, st["u"], st["rho"], None, self.grid.t)

    def synchronize(self):
        pass

    def download(self):
        return self.grid.download()


class LocalExchange:
    """Halo exchange between the slabs of one process (a ring in slab order)."""

    def __init__(self, slabs):
        self.slabs = slabs

    def exchange(self):
        R = len(self.slabs)
        for s in self.slabs:
            s.pack()
        for r, s in enumerate(self.slabs):
            s.recv[0].copy_(self.slabs[(r - 1) % R].send[1])   # left neighbour's last real plane
            s.recv[1].copy_(self.slabs[(r + 1) % R].send[0])   # right neighbour's first real plane
        for s in self.slabs:
            s.unpack()


class DistExchange:
    """Halo exchange of this rank's slab with the neighbouring ranks' slabs
    over torch.distributed point-to-point messages (a ring of ranks)."""

    def __init__(self, slab, rank: int, world: int, group=None):
        self.slab, self.rank, self.world, self.group = slab, rank, world, group

    def exchange(self):
        import torch.distributed as dist
        s = self.slab
        left, right = (self.rank - 1) % self.world, (self.rank + 1) % self.world
        s.pack()
        if self.world == 1:
            s.recv[0].copy_(s.send[1])
            s.recv[1].copy_(s.send[0])
        else:
            # With two ranks both neighbours are the same peer: the messages
            # are told apart by tag (1: travelling right, 0: travelling left)
            # and, for transports that match by order, by the same order on
            # every rank (the right-going send first, the receive from the
            # left first).
            ops = [dist.P2POp(dist.isend, s.send[1], right, self.group, tag=1),
                   dist.P2POp(dist.isend, s.send[0], left, self.group, tag=0),
                   dist.P2POp(dist.irecv, s.recv[0], left, self.group, tag=1),
                   dist.P2POp(dist.irecv, s.recv[1], right, self.group, tag=0)]
            for req in dist.batch_isend_irecv(ops):
                req.wait()
        s.unpack()


def run(slabs_or_slab, exchange, steps: int) -> None:
    """`steps` steps of the decomposed grid: step every slab, then exchange."""
    slabs = slabs_or_slab if isinstance(slabs_or_slab, list) else [slabs_or_slab]
    for _ in range(steps):
        for s in slabs:
            s.step(1)
        exchange.exchange()


def gather(l0, ranges, states, key: str, per_site: int) -> np.ndarray:
    """The global array `key` from the slabs' downloads (real planes only)."""
    out = np.empty((l0.N, l0.M * l0.K * per_site))
    for (a, b), st in zip(ranges, states):
        loc = st[key].reshape(b - a + 2, -1)
        out[a:b] = loc[1:-1]
    return out.reshape(-1)
