"""Shared helpers for the parity tests: rebuild an oracle case's level-0
description from ``cases.py`` and run it on a backend (oracle or GPU)."""
from __future__ import annotations

import hashlib
import os

import numpy as np

from luma_gb300 import bfl
from luma_gb300 import case as hostcase
from tests.golden import cases as CASES

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture(name: str) -> dict:
    with np.load(os.path.join(HERE, f"{name}.npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def level0(name: str) -> hostcase.Level0:
    spec = CASES.CASES[name]
    l0 = hostcase.build_level0(spec["defs"])
    init = CASES.initial_fields(name)
    if init is not None:
        l0.u = init["u"].copy()
    b = spec.get("bfl")
    if b:
        make = bfl.circle_body if spec["defs"].dims == 2 else bfl.sphere_body
        body = make(l0, b["centre"], b["radius"])
        l0.typ = body.typ
        l0.bfl = body
    return l0


def initial_state(l0: hostcase.Level0):
    d = l0.defs
    f0 = hostcase.equilibrium(d.dims, d.Q, l0.rho, l0.u).reshape(-1)
    return f0, l0.u.copy(), l0.rho.copy(), l0.force_xyz.copy()


def hierarchy(name: str) -> list:
    """[level0, level1, ...] of an oracle case (one region per level), built
    by the host set-up; parents are relabelled as children are added."""
    spec = CASES.CASES[name]
    grids = [level0(name)]
    for r in spec.get("regions", []):
        grids.append(hostcase.build_subgrid(grids[-1], r[0], r[1]))
    return grids


def grid_key(g) -> str:
    return f"L{g.level}R{g.region}"


def build_backend(name: str, make, precision=None):
    """Create the grid tree of an oracle case on a backend.

    `make(desc, parent)` builds one grid (OracleGrid or GpuGrid); returns
    (grids, levels) with each grid's initial state uploaded."""
    levels = hierarchy(name)
    grids = []
    for lv in levels:
        desc = lv.desc() if precision is None else lv.desc(precision=precision)
        g = make(desc, grids[-1] if grids else None)
        grids.append(g)
    for g, lv in zip(grids, levels):
        g.upload(*initial_state(lv), t=0)
        body = getattr(lv, "bfl", None)
        if body is not None:
            g.bfl_set(body.site_marker, body.q)
    return grids, levels


def fields_at(fx: dict, key: str, s: int, name: str):
    """(u, rho, u_sha, rho_sha, f_sha) of grid `key` at step s from a fixture."""
    pre = "" if key == "L0R0" else key + "_"
    return (fx.get(f"{pre}u_{s}"), fx.get(f"{pre}rho_{s}"), str(fx[f"{pre}u_sha_{s}"]),
            str(fx[f"{pre}rho_sha_{s}"]), str(fx[f"{pre}f_sha_{s}"]))


def grid_dm(lv) -> float:
    """GridObj::dm: (L_PHYSICAL_RHO / L_RHOIN) * dh^3 on L0, /8 per level."""
    d = lv.defs
    return (d.physical_rho / d.rho_in) * lv.dh * lv.dh * lv.dh


def attach_filaments(name, grids, levels, add):
    """Add the case's filaments with `add(grid, **params)` on level 0."""
    out = []
    for fl in CASES.CASES[name].get("filaments", []):
        lv = levels[0]
        out.append(add(grids[0], start=CASES.filament_start(name, fl), length=fl["length"], height=fl["height"],
                       depth=fl["depth"], angle_v=fl["angle_v"], nel=fl["nel"], clamped=fl["clamped"],
                       density=fl["density"], E=fl["E"], dm=grid_dm(lv),
                       fsi_vel_scale=lv.defs.ux0 * lv.dt / lv.dh))
    return out
