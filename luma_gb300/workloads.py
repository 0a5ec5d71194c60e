"""Synthetic workloads of the named shapes, built through the host set-up.

``sphere_refined``: D3Q19 BGK flow past a rigid IB sphere, base grid
384 x 192 x 192 with two embedded refinement levels (factor 2 each) in boxes
centred on the sphere; sphere diameter 24 base lattice units with a
Fibonacci (golden-angle) layout of 5000 markers; uniform inlet u = 0.04 lu,
Re = 100 on the diameter (nu = 0.04 * 24 / 100 in base lattice units).
Inlet: forced-equilibrium velocity face; outlet: extrapolate-right; lateral
faces periodic.

Where the body lives: 5000 markers on the sphere of 96 level-2 lattice
units (diameter) sit 2.4 lu apart, and the direct-forcing IBM (epsilon near
3.5) diverges within a few steps there, in the reference's arithmetic as in
this path (the oracle shows it on a scaled copy).  So the body is on level 1
(diameter 48 lu, markers 1.2 lu apart; the reference's geometry reader would
place 7238 there), and the level-2 box sits inside the sphere, centred on
it, clear of the markers' supports.

``run_sphere`` steps it on the GPU and reports MLUPS (fine updates counted
2^level times per base step, as the reference's activeCellOps counts them),
the drag coefficient from the FP64 marker-force sum, and the FP64/FP32
field difference when both are run.

``kbc_filaments``: D3Q27 KBC 512 x 256 x 256 with one refinement level
around an array of 64 FEM filaments (32 elements, one marker per node), the
filament-array workload; ``run_filaments`` steps it and reports MLUPS and
the filament tips.  The reference cannot run it (its FEM aborts in 3D); the
structure density is 100x the fluid's, since lighter filaments in the
reference's 3D coupling diverge within a few dozen steps (oracle, scaled
copy).

``bfl_cylinder``: D2Q9 BGK channel 8192 x 2048 (solid bottom/top, uniform
forced-equilibrium inlet u = 0.04 lu and the same initial velocity inside,
extrapolate-right outlet) with a
rigid BFL cylinder of radius 128 lu at 1/4 of the length, built as the
reference's CIRCLE_SPHERE BFL prefab (``bfl.circle_body``, with the closure's
projection count reset per closure: the reference's own count doubles per
closure marker and never finishes a circle this size); ``run_bfl``
steps it and reports MLUPS, the BFL link count and the body's
momentum-exchange force.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import _abi as A
from . import case as hostcase


def fibonacci_sphere(cx: float, cy: float, cz: float, radius: float, n: int) -> np.ndarray:
    """Golden-angle layout of n points on a sphere, (n, 3)."""
    inc = math.pi * (3.0 - math.sqrt(5.0))
    off = 2.0 / n
    k = np.arange(n)
    y = k * off - 1.0 + off / 2.0
    r = np.sqrt(1.0 - y * y)
    phi = k * inc
    return np.stack([cx + np.cos(phi) * r * radius, cy + y * radius, cz + np.sin(phi) * r * radius], axis=1)


def sphere_refined(nx: int = 384, ny: int = 192, nz: int = 192, diameter_lu: float = 24.0, n_markers: int = 5000,
                   u_lu: float = 0.04, re: float = 100.0, resolution: int = 16, l1_half: int = 24,
                   l2_half: int = 4, body_level: int = 1):
    """(levels [L0, L1, L2], markers (n, 3)) of the sphere workload.  The
    sphere centre is nx/4 base cells from the inlet on the lateral centre
    line; the level-1 box spans +-l1_half base cells around it, the level-2
    box +-l2_half.  The body lives on `body_level`."""
    dh = 1.0 / resolution
    dt = u_lu * dh                    # ux0 = 1: ux0 * dt / dh = u_lu
    nu_lbm = u_lu * diameter_lu / re
    nu = nu_lbm * dh * dh / dt        # L_NU: nu_lbm = nu * dt / dh^2
    V, X, F = A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.FLUID
    defs = hostcase.Definitions(dims=3, resolution=resolution, timestep=dt, bx=nx / resolution, by=ny / resolution,
                                bz=nz / resolution, re=None, nu=nu, ux0=1.0, no_flow=False, ibm=True,
                                walls=(V, X, F, F, F, F))
    l0 = hostcase.build_level0(defs)
    c = np.array([nx / 4.0, ny / 2.0, nz / 2.0]) * dh
    lo1, hi1 = tuple(c - l1_half * dh), tuple(c + l1_half * dh)
    l1 = hostcase.build_subgrid(l0, lo1, hi1)
    lo2, hi2 = tuple(c - l2_half * dh), tuple(c + l2_half * dh)
    l2 = hostcase.build_subgrid(l1, lo2, hi2)
    mk = fibonacci_sphere(c[0], c[1], c[2], 0.5 * diameter_lu * dh, n_markers)
    return [l0, l1, l2], mk


BODY_LEVEL = 1


def upload_level(g, lv) -> None:
    f0 = hostcase.equilibrium(lv.defs.dims, lv.defs.Q, lv.rho, lv.u).reshape(-1)
    g.upload(f0, lv.u, lv.rho, lv.force_xyz, 0)


def run_sphere(precision: int, steps: int, warmup: int = 5, stream=None, levels=None, markers=None,
               diameter_lu: float = 24.0, u_lu: float = 0.04, body_level: int = BODY_LEVEL,
               trace: str | None = None, trace_steps: int = 4) -> dict:
    """Steps the sphere workload; returns timing, Cd and the L0 fields.
    With `trace`, `trace_steps` further steps (after everything measured)
    are recorded as a kernel timeline to that path (luma_gb300.timeline)."""
    from .gpu import GpuGrid
    if levels is None:
        levels, markers = sphere_refined(diameter_lu=diameter_lu, u_lu=u_lu)
    grids = []
    for lv in levels:
        g = GpuGrid(lv.desc(precision=precision), grids[-1] if grids else None)
        if stream is not None:
            g.set_stream(stream)
        grids.append(g)
    for g, lv in zip(grids, levels):
        upload_level(g, lv)
    fine = grids[body_level]
    fine.ibm_add_body(markers)
    t = time.perf_counter()
    grids[0].ibm_initialise()
    t_init = time.perf_counter() - t
    grids[0].step(warmup)
    grids[0].synchronize()
    t = time.perf_counter()
    grids[0].step(steps)
    grids[0].synchronize()
    sec = time.perf_counter() - t
    lu = sum(lv.ncell * (2 ** lv.level) for lv in levels)
    F = fine.ibm_body_force(0)
    Dl = diameter_lu * 2 ** body_level             # diameter in the body level's lattice units
    cd = 2.0 * F[0] / (1.0 * u_lu * u_lu * math.pi * Dl * Dl / 4.0)
    st = grids[0].download(f=False)
    out = {"steps": steps, "warmup": warmup, "seconds": sec, "ms_per_step": sec / steps * 1e3,
           "mlups": lu * steps / sec / 1e6, "lattice_updates_per_step": lu, "cd": cd, "force": F.tolist(),
           "ibm_init_s": t_init, "u0": st["u"], "rho0": st["rho"],
           "sites": [lv.ncell for lv in levels], "markers": int(len(markers))}
    if trace:
        from . import timeline
        timeline.record(grids[0], trace_steps, trace)
    for g in reversed(grids):
        g.close()
    return out


def kbc_filaments(nx: int = 512, ny: int = 256, nz: int = 256, n_fil: int = 64, nel: int = 32, u_lu: float = 0.03,
                  re: float = 1000.0, resolution: int = 32, box=(96, 64, 96), ei_range=(1e-3, 1e-1),
                  density_ratio: float = 100.0, seed: int = 20261204):
    """(levels [L0, L1], filaments [dict of luma_gpu_ibm_add_filament
    arguments]) of the filament-array workload: D3Q27 KBC (streamed-population
    form), base grid nx x ny x nz, one refinement level in a box of `box` base
    cells centred in y and z and starting nx/4 from the inlet; n_fil
    filaments on level 1 on an 8 x 8 array over x-z with seeded jitter, each
    clamped at the box's lower third and pointing +y, nel elements, one
    marker per node (length nel level-1 lattice units), thickness and depth
    one level-1 lattice unit, structure density density_ratio x fluid.
    Bending rigidity EI log-uniform in ei_range, non-dimensional
    (EI / (rho U^2 L^3), L the filament length).  Uniform inlet u = u_lu,
    Re = u L / nu = re on the filament length; outlet extrapolate-right,
    bottom/top solid, front/back periodic."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dh = 1.0 / resolution
    dt = u_lu * dh
    dh1 = dh / 2.0
    L = nel * dh1                             # filament length (one marker per node)
    nu = 1.0 * L / re                         # L_NU with ux0 = 1
    V, X, S, F = A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.FLUID
    defs = hostcase.Definitions(dims=3, resolution=resolution, timestep=dt, bx=nx / resolution, by=ny / resolution,
                                bz=nz / resolution, re=None, nu=nu, ux0=1.0, no_flow=False, ibm=True, kbc=True,
                                walls=(V, X, S, S, F, F))
    l0 = hostcase.build_level0(defs)
    bx, by, bz = box
    x0 = (nx // 4) * dh
    y0 = (ny // 2 - by // 2) * dh
    z0 = (nz // 2 - bz // 2) * dh
    l1 = hostcase.build_subgrid(l0, (x0, y0, z0), (x0 + bx * dh, y0 + by * dh, z0 + bz * dh))
    side = int(round(math.sqrt(n_fil)))
    fils = []
    rho_f = defs.physical_rho
    dm = (rho_f / defs.rho_in) * dh1 ** 3
    h = dh1
    depth = dh1
    I = depth * h ** 3 / 12.0
    for q in range(n_fil):
        ix, iz = q % side, q // side
        px = x0 + (ix + 0.5 + rng.uniform(-0.25, 0.25)) * (bx * dh) / side
        pz = z0 + (iz + 0.5 + rng.uniform(-0.25, 0.25)) * (bz * dh) / side
        py = y0 + by * dh / 3.0
        ei = math.exp(rng.uniform(math.log(ei_range[0]), math.log(ei_range[1])))
        E = ei * rho_f * 1.0 * L ** 3 / I
        fils.append(dict(start=(px, py, pz), length=L, height=h, depth=depth, angle_v=90.0, nel=nel, clamped=True,
                         density=density_ratio * rho_f, E=E, dm=dm, fsi_vel_scale=1.0 * dt / dh1))
    return [l0, l1], fils


def run_filaments(precision: int, steps: int, warmup: int = 2, levels=None, fils=None, fix_kbc: bool = True,
                  trace: str | None = None, trace_steps: int = 4) -> dict:
    """Steps the filament-array workload; returns timing and tip positions.
    `trace` as for run_sphere."""
    from .gpu import GpuGrid
    if levels is None:
        levels, fils = kbc_filaments()
    grids = []
    for lv in levels:
        desc = lv.desc(precision=precision, fix_kbc=fix_kbc)
        g = GpuGrid(desc, grids[-1] if grids else None)
        grids.append(g)
    for g, lv in zip(grids, levels):
        upload_level(g, lv)
    fine = grids[-1]
    for fl in fils:
        fine.ibm_add_filament(**fl)
    t = time.perf_counter()
    grids[0].ibm_initialise()
    t_init = time.perf_counter() - t
    tip0 = np.array([fine.ibm_markers(b)[-1, :3] for b in range(len(fils))])
    grids[0].step(warmup)
    grids[0].synchronize()
    t = time.perf_counter()
    grids[0].step(steps)
    grids[0].synchronize()
    sec = time.perf_counter() - t
    lu = sum(lv.ncell * (2 ** lv.level) for lv in levels)
    tips = np.array([fine.ibm_markers(b)[-1, :3] for b in range(len(fils))])
    st = grids[0].download(f=False)
    out = {"steps": steps, "warmup": warmup, "seconds": sec, "ms_per_step": sec / steps * 1e3,
           "mlups": lu * steps / sec / 1e6, "lattice_updates_per_step": lu, "ibm_init_s": t_init,
           "tip0": tip0, "tips": tips, "u0": st["u"], "sites": [lv.ncell for lv in levels],
           "finite": bool(np.isfinite(st["u"]).all())}
    if trace:
        from . import timeline
        timeline.record(grids[0], trace_steps, trace)
    for g in reversed(grids):
        g.close()
    return out


def bfl_cylinder(nx: int = 8192, ny: int = 2048, radius_lu: float = 128.0, u_lu: float = 0.04,
                 re_d: float = 250.0):
    """(level0, BflBody) of the BFL channel workload; Re on the diameter."""
    from . import bfl
    res = ny // 2                               # the channel is 2 length units high
    dh = 1.0 / res
    nu_lu = u_lu * 2.0 * radius_lu / re_d
    defs = hostcase.Definitions(dims=2, resolution=res, timestep=u_lu * dh, bx=nx / res, by=2.0,
                                re=u_lu / (nu_lu * dh), ux0=1.0, no_flow=False,
                                walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    l0 = hostcase.build_level0(defs)
    body = bfl.circle_body(l0, (0.25 * nx * dh, 1.0 - dh, 0.0), radius_lu * dh, reset_projection=True)
    l0.typ = body.typ
    return l0, body


def run_bfl(precision: int, steps: int, warmup: int = 5, l0=None, body=None) -> dict:
    """Steps the BFL workload; returns timing, the body force and the fields."""
    from .gpu import GpuGrid
    if l0 is None:
        l0, body = bfl_cylinder()
    g = GpuGrid(l0.desc(precision=precision))
    upload_level(g, l0)
    g.bfl_set(body.site_marker, body.q)
    g.step(warmup)
    g.synchronize()
    t = time.perf_counter()
    g.step(steps)
    g.synchronize()
    sec = time.perf_counter() - t
    F = g.bfl_forces().sum(axis=0)
    st = g.download(f=False)
    g.close()
    return {"steps": steps, "warmup": warmup, "seconds": sec, "ms_per_step": sec / steps * 1e3,
            "mlups": l0.ncell * steps / sec / 1e6, "sites": l0.ncell, "markers": int(len(body.positions)),
            "links": int((body.q >= 0).sum()), "force": F.tolist(), "u": st["u"], "rho": st["rho"]}
