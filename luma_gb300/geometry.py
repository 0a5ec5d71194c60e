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

* ``FROM_FILE BBB|BFL|IBM file lev reg START|CENTRE x START|CENTRE y
  START|CENTRE z length X|Y|Z RIGID|MOVABLE CLAMPED|SUPPORTED`` (:360-452
  with ``io_readInCloud``, :812-1058): the point cloud scaled to `length`
  along the direction and placed at the reference position, kept where it
  lies on the grid; BBB labels the fluid sites enclosing the points solid
  (``addBouncebackObject``, src/ObjectManager.cpp:304-338: u set to 0 with
  the 3D quirk that sets u_x twice and leaves u_z, rho to L_RHOIN); BFL and
  IBM bodies take the voxel-grid filter's markers (``Body::buildFromCloud``
  / ``passToVoxelFilter``, inc/Body.h:622-790).

The prefab entries shift positions by the solid-wall thickness as the
reader does (left, bottom, front walls); FROM_FILE does not.  The reader
skips '#' lines only at the top of the file; so does this.
"""
from __future__ import annotations

import math

from . import _abi as A
from . import bfl as _bfl
from . import case as _case


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


L_SMALL_NUMBER = 1e-8


_cround = _case.cround  # std::round


def read_cloud(text: str, dims: int) -> list:
    """Points of a cloud file as io_readInCloud reads them: one "x y z" line
    each (z forced to 0 in 2D); a line without values (the empty line after
    a final newline) repeats the previous point, as the reader's stream
    extraction leaves its variables unchanged."""
    pts = []
    x = y = z = None
    for line in text.split("\n"):
        vals = line.split()
        if len(vals) > 0:
            x = float(vals[0])
        if len(vals) > 1:
            y = float(vals[1])
        if len(vals) > 2:
            z = float(vals[2])
        if x is None or y is None or (dims == 3 and z is None):
            # the reference would store uninitialised values here
            raise ValueError("cloud file: a point before any complete coordinates")
        pts.append((x, y, z if dims == 3 else 0.0))
    return pts


def place_cloud(lv, pts, refs, length: float, direction: str) -> list:
    """Scale and shift a cloud as io_readInCloud does (:850-1000) and keep
    the points that lie on the grid; `refs` = ((centre?, value) per axis)."""
    D = lv.defs.dims
    dcell = lv.dh
    ref = [_cround(r / dcell) * dcell for _, r in refs]
    blen = _cround(length / dcell) * dcell
    axes = [[p[a] for p in pts] for a in range(3)]
    ai = "XYZ".index(direction)
    scale = (blen - 2 * L_SMALL_NUMBER * dcell) / abs(max(axes[ai]) - min(axes[ai]))
    shift = [0.0, 0.0, 0.0]
    for a in range(3):
        lo, hi = min(axes[a]), max(axes[a])
        if refs[a][0]:
            ref[a] += (dcell / 2.0)
            dist = scale * abs(hi - lo)
            dist = _cround(dist / dcell) * dcell
            start = ref[a] - (dist / 2.0)
            shift[a] = start - scale * lo
        else:
            shift[a] = (ref[a] + L_SMALL_NUMBER * dcell) - scale * lo
    E = lv.global_edges
    out = []
    for p in pts:
        x = p[0] * scale
        x += shift[0]
        y = p[1] * scale
        y += shift[1]
        z = p[2]
        if D == 3:
            z = z * scale
            z += shift[2]
        v = _voxel(lv, x, y, z)
        inside = E[0] <= x < E[1] and E[2] <= y < E[3] and (D != 3 or E[4] <= z < E[5])
        if inside and v is not None:
            out.append((x, y, z))
    return out


def _voxel(lv, x, y, z):
    """GridUtils::getEnclosingVoxel on the grid's own edges, None off the
    grid (isOffGrid)."""
    D = lv.defs.dims
    e = lv.edges if lv.edges is not None else lv.global_edges
    v = (int(math.floor((x - e[0]) / lv.dh)), int(math.floor((y - e[2]) / lv.dh)),
         int(math.floor((z - e[4]) / lv.dh)) if D == 3 else 0)
    if not (0 <= v[0] < lv.N and 0 <= v[1] < lv.M and 0 <= v[2] < lv.K):
        return None
    return v


def voxel_filter(lv, pts) -> tuple:
    """Body::buildFromCloud: one marker per voxel at the running mean of the
    points that fall in it, in the reference's order (the current marker's
    voxel window first, then any earlier marker's voxel, else a new
    marker).  Returns (positions, voxels, first points): a marker's primary
    support voxel and IBMarker::position0 stay those of the point that made
    it."""
    pos, vox, count, made = [], [], [], []
    first = {}
    half = lv.dh / 2.0
    E = lv.global_edges
    D = lv.defs.dims

    def add(i, p):
        v = _voxel(lv, *p)
        made.append(i)
        pos.append(list(p))
        vox.append(v)
        count.append(1)
        first.setdefault(v, len(pos) - 1)

    def mean(m, p):
        count[m] += 1
        c = count[m]
        for a in range(3):
            pos[m][a] = ((pos[m][a] * (c - 1)) + p[a]) / c

    add(0, pts[0])
    cur = 0
    for i, p in enumerate(pts[1:], 1):
        vx, vy, vz = lv.xpos[vox[cur][0]], lv.ypos[vox[cur][1]], lv.zpos[vox[cur][2]]
        if (vx - half <= p[0] < vx + half) and (vy - half <= p[1] < vy + half) and (vz - half <= p[2] < vz + half):
            mean(cur, p)
            continue
        inside = E[0] <= p[0] < E[1] and E[2] <= p[1] < E[3] and (D != 3 or E[4] <= p[2] < E[5])
        v = _voxel(lv, *p) if inside else None
        if v is not None and v in first:
            cur = first[v]
            mean(cur, p)
            continue
        cur = len(count)
        add(i, p)
    return [tuple(q) for q in pos], vox, [tuple(pts[i]) for i in made]


def _rigid(btype, move, lev, reg, lv, pts) -> dict:
    if btype == "IBM":
        if move == "FLEXIBLE":
            raise NotImplementedError("flexible bodies other than filaments")
        return {"kind": "ibm", "level": int(lev), "region": int(reg), "movable": move == "MOVABLE",
                "positions": pts}
    if btype == "BFL":
        return {"kind": "bfl", "level": int(lev), "region": int(reg), "body": _bfl._build(lv, pts, False)}
    raise NotImplementedError(f"boundary type {btype}")


def read_geometry(text: str, levels: dict, dm=None, ux0: float | None = None, clouds: dict | None = None) -> list:
    """Bodies of a geometry.config text.

    ``levels`` maps (level, region) to the grid's host description
    (``case.Level0`` or a sub-grid); ``dm(lv)`` gives a grid's
    ``GridObj::dm`` for filaments (default (L_PHYSICAL_RHO / L_RHOIN) dh^3).
    ``clouds`` maps a FROM_FILE entry's file name to the file's text.
    Returns dicts with ``kind`` "ibm" (``positions``, ``movable``), "bfl"
    (``body``, a ``bfl.BflBody``), "filament" (the keyword arguments of
    ``GpuGrid.ibm_add_filament``) or "bbb" (``sites`` to label, see
    ``apply_bbb``), each with ``level`` and ``region``, in the reader's body
    order."""
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
        elif case == "FROM_FILE":
            (btype, fname, lev, reg, xrt, xr, yrt, yr, zrt, zr, length, direction, move, bc) = take(14)
            if int(lev) < 0:
                raise NotImplementedError("FROM_FILE bodies spanning levels (level -1)")
            if btype not in ("BBB", "BFL", "IBM"):
                raise ValueError(f"FROM_FILE: unknown boundary type {btype}")
            if direction not in ("X", "Y", "Z"):
                raise ValueError(f"FROM_FILE: unknown scale direction {direction}")
            lv = grid(lev, reg)
            if clouds is None or fname not in clouds:
                raise ValueError(f"geometry config: no cloud text for {fname}")
            for rt in (xrt, yrt, zrt):
                if rt not in ("START", "CENTRE"):
                    raise ValueError(f"Unknown reference type {rt}")
            pts = place_cloud(lv, read_cloud(clouds[fname], lv.defs.dims),
                              ((xrt == "CENTRE", float(xr)), (yrt == "CENTRE", float(yr)), (zrt == "CENTRE", float(zr))),
                              float(length), direction)
            if not pts:
                continue  # nothing of the body on the grid
            if btype == "BBB":
                out.append({"kind": "bbb", "level": int(lev), "region": int(reg),
                            "sites": [_voxel(lv, *q) for q in pts]})
                continue
            if btype == "IBM" and move == "FLEXIBLE":
                raise NotImplementedError("flexible bodies other than filaments")
            mk, vox, p0 = voxel_filter(lv, pts)
            if btype == "IBM":
                out.append({"kind": "ibm", "level": int(lev), "region": int(reg),
                            "movable": move == "MOVABLE", "positions": mk, "positions0": p0})
            else:
                out.append({"kind": "bfl", "level": int(lev), "region": int(reg),
                            "body": _bfl._build(lv, mk, False, voxels=vox)})
        else:
            raise NotImplementedError(f"geometry entry {case}")
    return out


def apply_bbb(lv, entry) -> None:
    """Label a BBB entry's sites solid on a host grid description as
    addBouncebackObject does: fluid sites only; u set to 0 (in 3D u_x twice,
    u_z kept) and rho to L_RHOIN.  The reference has set the populations
    from u and rho when it built the grid, before it reads the geometry:
    take them from the description before labelling to match."""
    N, M, K = lv.N, lv.M, lv.K
    D = lv.defs.dims
    typ = lv.typ.reshape(N, M, K).copy()
    u = lv.u.reshape(N, M, K, D).copy()
    rho = lv.rho.reshape(N, M, K).copy()
    for (i, j, k) in entry["sites"]:
        if typ[i, j, k] == A.FLUID:
            typ[i, j, k] = A.SOLID
            u[i, j, k, 0] = 0.0
            u[i, j, k, 1] = 0.0
            if D == 3:
                u[i, j, k, 0] = 0.0
            rho[i, j, k] = lv.defs.rho_in
    lv.typ = typ.reshape(-1)
    lv.u = u.reshape(-1)
    lv.rho = rho.reshape(-1)
