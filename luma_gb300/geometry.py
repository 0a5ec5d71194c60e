"""Host restatement of the geometry reader for the bodies this path builds.

``ObjectManager::io_readInGeomConfig`` (LUMA src/ObjectManager_ops_io.cpp:
322-800) turns ``input/geometry.config`` into bodies.  ``read_geometry``
parses the same text for:

* ``CIRCLE_SPHERE IBM|BFL lev reg x y z radius RIGID|MOVABLE`` (:570-631):
  an IB body at the prefab's marker positions (``prefab_points``), or a BFL
  body set up as the reference's BFLBody does (``bfl.circle_body`` /
  ``bfl.sphere_body``);
* ``FILAMENT_ARRAY IBM lev reg n x y z dx dy dz length height depth
  angle_v angle_h FLEXIBLE nel|CONFORMING CLAMPED|SUPPORTED density E``
  (:455-567): n flexible FEM filaments at start + i (dx, dy, dz), the
  arguments of ``luma_gpu_ibm_add_filament``.

Both shift positions by the solid-wall thickness as the reader does (left,
bottom, front walls).  The reader skips '#' lines only at the top of the
file; so does this.  Other entries (FROM_FILE point clouds, SQUARE_CUBE,
PLATE, rigid filaments) raise ``NotImplementedError`` naming the entry.
"""
from __future__ import annotations

import math

from . import _abi as A
from . import bfl as _bfl


def _shift(lv) -> tuple:
    d = lv.defs
    wt = lv.wall_thickness
    return (wt[0] if d.walls[0] == A.SOLID else 0.0, wt[2] if d.walls[2] == A.SOLID else 0.0,
            wt[4] if d.walls[4] == A.SOLID else 0.0)


prefab_points = _bfl.prefab_points


def read_geometry(text: str, levels: dict, dm=None, ux0: float | None = None) -> list:
    """Bodies of a geometry.config text.

    ``levels`` maps (level, region) to the grid's host description
    (``case.Level0`` or a sub-grid); ``dm(lv)`` gives a grid's
    ``GridObj::dm`` for filaments (default (L_PHYSICAL_RHO / L_RHOIN) dh^3).
    Returns dicts with ``kind`` "ibm" (``positions``, ``movable``), "bfl"
    (``body``, a ``bfl.BflBody``) or "filament" (the keyword arguments of
    ``GpuGrid.ibm_add_filament``), each with ``level`` and ``region``, in
    the reader's body order."""
    lines = text.split("\n")
    while lines and lines[0].startswith("#"):
        lines = lines[1:]
    tok = " ".join(lines).split()
    out = []
    p = 0

    def take(n):
        nonlocal p
        if p + n > len(tok):
            raise ValueError("geometry config: entry cut short")
        vals = tok[p:p + n]
        p += n
        return vals

    def grid(lev, reg):
        key = (int(lev), int(reg))
        if key not in levels:
            raise ValueError(f"geometry config: no grid level {key[0]} region {key[1]}")
        return levels[key]

    def default_dm(lv):
        d = lv.defs
        return (d.physical_rho / d.rho_in) * lv.dh * lv.dh * lv.dh

    while p < len(tok):
        case = take(1)[0]
        if case == "CIRCLE_SPHERE":
            btype, lev, reg, x, y, z, r, move = take(8)
            lv = grid(lev, reg)
            centre = (float(x), float(y), float(z))
            if move == "FLEXIBLE":
                raise ValueError("Circle/sphere cannot be flexible")
            if btype == "IBM":
                out.append({"kind": "ibm", "level": int(lev), "region": int(reg), "movable": move == "MOVABLE",
                            "positions": prefab_points(lv, centre, float(r))})
            elif btype == "BFL":
                make = _bfl.sphere_body if lv.defs.dims == 3 else _bfl.circle_body
                out.append({"kind": "bfl", "level": int(lev), "region": int(reg),
                            "body": make(lv, centre, float(r))})
            else:
                raise NotImplementedError(f"CIRCLE_SPHERE {btype}")
        elif case == "FILAMENT_ARRAY":
            (btype, lev, reg, n, sx, sy, sz, dx, dy, dz, length, height, depth, av, ah, move, nel, bc, rho,
             E) = take(20)
            if btype != "IBM" or move != "FLEXIBLE":
                raise NotImplementedError(f"FILAMENT_ARRAY {btype} {move}")
            lv = grid(lev, reg)
            shift = _shift(lv)
            start = (float(sx) + shift[0], float(sy) + shift[1], float(sz) + shift[2])
            space = (float(dx), float(dy), float(dz))
            nel_i = int(math.floor(float(length) / lv.dh)) if nel == "CONFORMING" else int(float(nel))
            D = lv.defs.dims
            u0 = lv.defs.ux0 if ux0 is None else ux0
            for i in range(int(n)):
                pos = [0.0, 0.0, 0.0]
                for d in range(D):
                    pos[d] = start[d] + i * space[d]
                out.append({"kind": "filament", "level": int(lev), "region": int(reg),
                            "args": dict(start=tuple(pos), length=float(length), height=float(height),
                                         depth=float(depth), angle_v=float(av), nel=nel_i,
                                         clamped=bc == "CLAMPED", density=float(rho), E=float(E),
                                         dm=(dm or default_dm)(lv), fsi_vel_scale=u0 * lv.dt / lv.dh)})
            del ah  # the planar beam has no horizontal angle
        else:
            raise NotImplementedError(f"geometry entry {case}")
    return out
