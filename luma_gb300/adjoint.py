"""Time-averaged drag of an immersed body and its discrete adjoint.

Python side of ``luma_gpu_adj_forward`` / ``luma_gpu_adj_backward``: the
objective is J = (1/T) sum_t sum_m F_m,x eps_m ds_m (* ds_m in 3D), the
lattice-unit drag that ObjectManager::io_writeLiftDrag integrates
(LUMA src/ObjectManager_ops_io.cpp:105-121), averaged over T steps.  Its
parameters are the scale s of the velocity of every inlet (velocity) site and
the body's marker positions.  ``DragFunction`` gives the pair the contract of
a ``torch.autograd.Function``: forward runs the checkpointed device forward,
backward the hand-written reverse sweep.

``cylinder_channel`` builds the D2Q9 channel with a circular cylinder of
markers on seeded, perturbed radii (the adjoint workload: 400 x 160 nodes,
diameter 20 lattice units, 64 markers, sigma 0.1 lattice units).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from . import case as hostcase

SEED = 20261204


@dataclass
class DragCase:
    defs: hostcase.Definitions
    markers: np.ndarray            # (n, 3) marker positions, reference length units
    nsteps: int
    checkpoint_every: int


def cylinder_markers(cx: float, cy: float, radius_lu: float, dh: float, n: int, sigma_lu: float,
                     seed: int = SEED) -> np.ndarray:
    """n markers at angles 2 pi i / n on radii radius_lu + N(0, sigma_lu^2)
    lattice units (PCG64 seeded), positions in length units."""
    rng = np.random.Generator(np.random.PCG64(seed))
    radii = (radius_lu + rng.normal(0.0, sigma_lu, size=n)) * dh
    th = 2.0 * math.pi * np.arange(n) / n
    return np.stack([cx + radii * np.cos(th), cy + radii * np.sin(th), np.zeros(n)], axis=1)


def cylinder_channel(nx: int = 400, ny: int = 160, diameter_lu: float = 20.0, n_markers: int = 64,
                     sigma_lu: float = 0.1, timestep: float = 1.0 / 2400.0, re: float = 100.0,
                     nsteps: int = 4000, checkpoint_every: int = 100, seed: int = SEED) -> DragCase:
    """D2Q9 BGK channel nx x ny: parabolic velocity inlet, extrapolate-right
    outlet, bounce-back walls top and bottom, fluid at rest initially; a
    rigid cylinder centred ny/2 lattice units from the inlet on the channel's
    centre line.  The length unit is half the channel height (resolution
    ny/2) and L_UX0 = 1, so the inlet's centre-line speed is
    u_max = 1.5 * timestep * resolution lattice units (0.05 by default);
    `re` is L_RE over that unit."""
    resolution = ny // 2                      # channel height = 2 length units
    bx, by = nx / resolution, ny / resolution
    V, X, S = A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID
    defs = hostcase.Definitions(dims=2, resolution=resolution, timestep=timestep, bx=bx, by=by, re=re, ux0=1.0,
                                parabolic_inlet=True, ibm=True, walls=(V, X, S, S, A.FLUID, A.FLUID))
    dh = 1.0 / resolution
    cx, cy = by / 2.0, by / 2.0
    mk = cylinder_markers(cx, cy, diameter_lu / 2.0, dh, n_markers, sigma_lu, seed)
    return DragCase(defs, mk, nsteps, checkpoint_every)


def inlet_u_max(c: DragCase) -> float:
    """Centre-line speed of the parabolic inlet profile (lattice units)."""
    return 1.5 * c.defs.ux0 * c.defs.timestep * c.defs.resolution


def initial_state(defs: hostcase.Definitions, inlet_scale: float = 1.0):
    """(level0, f, u, rho) with the velocity of every velocity site scaled."""
    l0 = hostcase.build_level0(defs)
    D = defs.dims
    u = l0.u.copy().reshape(-1, D)
    u[np.asarray(l0.typ) == A.VELOCITY] *= inlet_scale
    u = u.reshape(-1)
    f0 = hostcase.equilibrium(defs.dims, defs.Q, l0.rho, l0.u).reshape(-1)
    return l0, f0, u, l0.rho.copy()


def make_grid(c: DragCase, precision: int, inlet_scale: float = 1.0, markers: np.ndarray | None = None):
    """A GpuGrid of the case with its body added and initialised."""
    from .gpu import GpuGrid
    l0, f0, u, rho = initial_state(c.defs, inlet_scale)
    g = GpuGrid(l0.desc(precision=precision))
    g.upload(f0, u, rho, l0.force_xyz.copy() if l0.force_xyz is not None else None, t=0)
    g.ibm_add_body(c.markers if markers is None else markers)
    g.ibm_initialise()
    return g, l0


def drag_and_gradient(c: DragCase, precision: int = A.PREC_FP64, inlet_scale: float = 1.0,
                      markers: np.ndarray | None = None, backward: bool = True):
    """(J, dJ/ds, dJ/dX (n, dims)) on the GPU; gradients None without backward."""
    g, _ = make_grid(c, precision, inlet_scale, markers)
    try:
        J = g.adj_forward(c.nsteps, c.checkpoint_every, 0)
        if not backward:
            return J, None, None
        gs, gx = g.adj_backward(1.0)
        return J, gs, gx
    finally:
        g.close()


def _torch_function():
    import torch

    class DragFunction(torch.autograd.Function):
        """J(inlet_scale, markers) with the device adjoint as its backward.

        forward(ctx, inlet_scale: 0-d tensor, markers: (n, 3) tensor, case,
        precision) -> 0-d FP64 tensor; backward returns dJ/ds and dJ/dX (the
        z column zero in 2D)."""

        @staticmethod
        def forward(ctx, inlet_scale, markers, case: DragCase, precision: int = A.PREC_FP64):
            mk = markers.detach().to("cpu", torch.float64).numpy()
            g, _ = make_grid(case, precision, float(inlet_scale), mk)
            J = g.adj_forward(case.nsteps, case.checkpoint_every, 0)
            ctx.grid = g
            ctx.dims = case.defs.dims
            ctx.shape = markers.shape
            ctx.device, ctx.dtype = markers.device, markers.dtype
            return torch.tensor(J, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gJ):
            g = ctx.grid
            try:
                gs, gx = g.adj_backward(float(gJ))
            finally:
                g.close()
                ctx.grid = None
            full = np.zeros(ctx.shape)
            full[:, :ctx.dims] = gx
            return (torch.tensor(gs, dtype=torch.float64),
                    torch.from_numpy(full).to(ctx.device, ctx.dtype), None, None)

    return DragFunction


def drag_function():
    """The torch.autograd.Function wrapper (imports torch on first use)."""
    global _DRAG_FN
    try:
        return _DRAG_FN
    except NameError:
        _DRAG_FN = _torch_function()
        return _DRAG_FN
