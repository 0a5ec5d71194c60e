"""Host restatement of the geometry reader for the bodies this path builds.

``ObjectManager::io_readInGeomConfig`` (LUMA src/ObjectManager_ops_io.cpp:
322-800) turns ``input/geometry.config`` into bodies.  ``read_geometry``
parses the same text for:

* ``CIRCLE_SPHERE IBM|BFL lev reg x y z radius RIGID|MOVABLE`` (:570-631):
  an IB body at the prefab's marker positions (``prefab_points``), or a BFL
  body set up as the reference's BFLBody does (``bfl.circle_body`` /
  ``bfl.sphere_body``);
* ``FILAMENT_ARRAY IBM|BFL lev reg n x y z dx dy dz length height depth
  angle_v angle_h FLEXIBLE|RIGID|MOVABLE nel|CONFORMING CLAMPED|SUPPORTED
  density E`` (:455-567): n filaments at start + i (dx, dy, dz) (in 2D the
  z of each start is 0, as the reader sets only the first L_DIMS
  components); flexible IB filaments as the arguments of
  ``luma_gpu_ibm_add_filament``, rigid/movable IB and BFL filaments at the
  filament prefab's points (``filament_points``);
* ``SQUARE_CUBE IBM|BFL lev reg x y z length height depth angle_v angle_h
  RIGID|MOVABLE`` (:636-710) at ``square_points``;
* ``PLATE IBM|BFL lev reg x y z length width angle_x angle_y angle_z
  RIGID|MOVABLE`` (3D, :711-790) at ``plate_points``.

All shift positions by the solid-wall thickness as the reader does (left,
bottom, front walls).  The reader skips '#' lines only at the top of the
file; so does this.  FROM_FILE point clouds raise ``NotImplementedError``.
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

_DEG = _bfl.L_PI / 180  # the reference's angle * L_PI / 180


def filament_points(lv, start, length: float, angle_v: float) -> list:
    """Filament prefab (``inc/Body.h:139-186``): floor(length / dh) + 1
    markers along the vertical angle.  Its horizontal angle is read under
    ``#if (L_DIM == 3)`` (a misspelt macro), so it is always 0."""
    n = int(math.floor(length / lv.dh)) + 1
    spacing = length / (n - 1)
    spacing_h = spacing * math.cos(angle_v * _bfl.L_PI / 180)
    ah = 0.0
    return [(start[0] + i * spacing_h * math.cos(ah * _bfl.L_PI / 180.0),
             start[1] + i * spacing * math.sin(angle_v * _bfl.L_PI / 180.0),
             start[2] + i * spacing_h * math.sin(ah * _bfl.L_PI / 180.0)) for i in range(n)]


def square_points(lv, centre, length: float, height: float, depth: float, angles) -> list:
    """Square/cuboid prefab (``inc/Body.h:258-395``): the surface points of
    a floor(l / dh) + 1 lattice per side, rotated by the vertical (and, in
    3D, horizontal) angle about the centre."""
    nl = int(math.floor(length / lv.dh)) + 1
    nh = int(math.floor(height / lv.dh)) + 1
    nd = int(math.floor(depth / lv.dh)) + 1
    D = lv.defs.dims
    total = nl * nh * nd - (nl - 2) * (nh - 2) * (nd - 2) if D == 3 else nl * nh - (nl - 2) * (nh - 2)
    if total < (24 if D == 3 else 8):
        raise ValueError("Resolution not high enough to build square/cuboid this small")
    sl, sh = length / (nl - 1), height / (nh - 1)
    sd = depth / (nd - 1) if nd > 1 else 0.0
    a0, a1 = angles[0] * _bfl.L_PI / 180, angles[1] * _bfl.L_PI / 180
    pts = []
    for i in range(nl):
        for j in range(nh):
            for k in (range(nd) if D == 3 else (0,)):
                x = -length / 2.0 + i * sl
                y = -height / 2.0 + j * sh
                if D == 3:
                    z = -depth / 2.0 + k * sd
                    if not (i in (0, nl - 1) or j in (0, nh - 1) or k in (0, nd - 1)):
                        continue
                    xd = (x * math.cos(a0) - y * math.sin(a0)) * math.cos(a1) - z * math.sin(a1)
                    yd = (y * math.cos(a0) + x * math.sin(a0))
                    zd = (x * math.cos(a0) - y * math.sin(a0)) * math.sin(a1) + z * math.cos(a1)
                else:
                    z = 0.0
                    if not (i in (0, nl - 1) or j in (0, nh - 1)):
                        continue
                    xd = x * math.cos(a0) - y * math.sin(a0)
                    yd = x * math.sin(a0) + y * math.cos(a0)
                    zd = z
                pts.append((xd + centre[0], yd + centre[1], zd + centre[2]))
    return pts


def _matvec(A, x):
    out = [0.0, 0.0, 0.0]
    for r in range(3):
        for c in range(3):
            out[r] += A[r][c] * x[c]
    return out


def plate_points(lv, centre, length: float, width: float, angles) -> list:
    """Plate prefab (3D, ``inc/Body.h:397-493``): a floor(l / dh) + 1 by
    floor(w / dh) + 1 lattice in the x-z plane rotated by Tz then Tx (the
    reference builds the y rotation into a matrix it never applies)."""
    nl = int(math.floor(length / lv.dh)) + 1
    nw = int(math.floor(width / lv.dh)) + 1
    sl, sw = length / (nl - 1), width / (nw - 1)
    tx, tz = angles[0] * _bfl.L_PI / 180.0, angles[2] * _bfl.L_PI / 180.0
    Tx = [[1.0, 0.0, 0.0], [0.0, math.cos(tx), -math.sin(tx)], [0.0, math.sin(tx), math.cos(tx)]]
    Tz = [[math.cos(tz), -math.sin(tz), 0.0], [math.sin(tz), math.cos(tz), 0.0], [0.0, 0.0, 1.0]]
    pts = []
    for i in range(nl):
        for j in range(nw):
            p = [-length / 2.0 + i * sl, 0.0, -width / 2.0 + j * sw]
            p = _matvec(Tx, _matvec(Tz, p))
            pts.append((p[0] + centre[0], p[1] + centre[1], p[2] + centre[2]))
    return pts


def _rigid(btype, move, lev, reg, lv, pts) -> dict:
    if btype == "IBM":
        if move == "FLEXIBLE":
            raise NotImplementedError("flexible bodies other than filaments")
        return {"kind": "ibm", "level": int(lev), "region": int(reg), "movable": move == "MOVABLE",
                "positions": pts}
    if btype == "BFL":
        return {"kind": "bfl", "level": int(lev), "region": int(reg), "body": _bfl._build(lv, pts, False)}
    raise NotImplementedError(f"boundary type {btype}")


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
        elif case in ("SQUARE_CUBE", "PLATE"):
            if case == "SQUARE_CUBE":
                btype, lev, reg, x, y, z, length, height, depth, av, ah, move = take(12)
            else:
                btype, lev, reg, x, y, z, length, width, ax, ay, az, move = take(12)
            lv = grid(lev, reg)
            sh = _shift(lv)
            centre = (float(x) + sh[0], float(y) + sh[1], float(z) + sh[2])
            if case == "SQUARE_CUBE":
                pts = square_points(lv, centre, float(length), float(height), float(depth), (float(av), float(ah)))
            else:
                if lv.defs.dims != 3:
                    raise ValueError("Can't build plate in 2D")
                pts = plate_points(lv, centre, float(length), float(width), (float(ax), float(ay), float(az)))
            out.append(_rigid(btype, move, lev, reg, lv, pts))
        elif case == "FILAMENT_ARRAY":
            (btype, lev, reg, n, sx, sy, sz, dx, dy, dz, length, height, depth, av, ah, move, nel, bc, rho,
             E) = take(20)
            lv = grid(lev, reg)
            if not (btype == "IBM" and move == "FLEXIBLE"):
                shift = _shift(lv)
                start = (float(sx) + shift[0], float(sy) + shift[1], float(sz) + shift[2])
                for i in range(int(n)):
                    pos = [0.0, 0.0, 0.0]
                    for d in range(lv.defs.dims):
                        pos[d] = start[d] + i * (float(dx), float(dy), float(dz))[d]
                    out.append(_rigid(btype, move, lev, reg, lv,
                                      filament_points(lv, pos, float(length), float(av))))
                continue
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
