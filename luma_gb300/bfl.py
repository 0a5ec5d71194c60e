"""Host set-up of BFL (Bouzidi-Firdaouss-Lallemand) bodies: the data the
device stream needs, built the way the reference's BFLBody builds it.

A BFL body is a set of markers, at most one looked up per lattice voxel.
The device step reads, per site, the marker whose voxel the site is
(``Body::getMarkerData``, LUMA ``inc/Body.h:581-614``: the first marker whose
primary support voxel matches) and, per marker, the link distances
``Q[v + Q*m]`` (``BFLBody::Q``; -1 where no wall cuts the link).

``circle_body`` (2D) and ``sphere_body`` (3D) follow:
  * the prefab ``Body(g, id, centre, radius)`` (``inc/Body.h:197-255``): in
    2D floor(2 pi r / dh) angles from ``GridUtils::linspace``, the first
    dropped; in 3D floor(4 pi r^2 / dh^2) Fibonacci points;
  * ``Marker`` voxels (``inc/Marker.h:66-95`` through
    ``GridUtils::getEnclosingVoxel``, ``src/GridUtils.cpp:1630-1718``);
  * ``BFLBody::initialise`` (``src/BFLBody.cpp:49-142``): eBFL labels, then
    ``enforceSurfaceClosure`` (``:548-715``), then ``computeQ`` over the eBFL
    sites in (i, j, k) order (2D overload ``:412-515``, 3D ``:244-404``).
The geometry reader shifts the centre by the solid-wall thickness
(``src/ObjectManager_ops_io.cpp:585-597``); both take the centre as written
in the geometry file and apply that shift.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from .case import lattice

L_PI = 3.14159265358979323846  # the reference's L_PI (inc/stdafx.h:114)


@dataclass
class BflBody:
    typ: np.ndarray          # (N*M*K,) int32 site labels with eBFL sites
    site_marker: np.ndarray  # (N*M*K,) int32, marker of the site's voxel or -1
    q: np.ndarray            # (nm, Q) link distances, -1 for none
    positions: np.ndarray    # (nm, 3)


def _linspace(lo: float, hi: float, n: int) -> list:
    n = max(n, 2)
    spacing = (hi - lo) / float(n - 1)
    return [lo + spacing * i for i in range(n)]


def _dot(a, b) -> float:
    s = 0.0
    for x, y in zip(a, b):
        s += x * y
    return s


def _vecnorm(v) -> float:
    s = 0.0
    for x in v:
        s += x * x
    return math.sqrt(s)


def prefab_points(lv, centre, radius: float) -> list:
    """Marker positions of the circle/sphere prefab (``inc/Body.h:197-255``)
    for a centre as written in the geometry file (the wall shift applied):
    in 2D floor(2 pi r / dh) angles from ``GridUtils::linspace``, the first
    dropped; in 3D floor(4 pi r^2 / dh^2) Fibonacci points."""
    d = lv.defs
    wt = lv.wall_thickness
    cx = centre[0] + (wt[0] if d.walls[0] == A.SOLID else 0.0)
    cy = centre[1] + (wt[2] if d.walls[2] == A.SOLID else 0.0)
    cz = centre[2] + (wt[4] if d.walls[4] == A.SOLID else 0.0)
    if d.dims == 3:
        n = int(math.floor(4.0 * L_PI * (radius ** 2) / (lv.dh ** 2)))
        inc = L_PI * (3 - math.sqrt(5))
        off = 2.0 / float(n)
        pts = []
        for k in range(n):
            y = k * off - 1 + (off / 2)
            r = math.sqrt(1 - y * y)
            phi = k * inc
            pts.append((cx + (math.cos(phi) * r * radius), y * radius + cy, cz + (math.sin(phi) * r * radius)))
        return pts
    n = int(math.floor(2.0 * L_PI * radius / lv.dh))
    theta = _linspace(0.0, 2.0 * L_PI - (2.0 * L_PI / float(n)), n)
    return [(cx + radius * math.cos(t), cy + radius * math.sin(t), cz) for t in theta[1:]]


def circle_body(level0, centre, radius: float, reset_projection: bool = False) -> BflBody:
    """A rigid 2D BFL circle on level 0 (reference ``CIRCLE_SPHERE BFL``).

    The reference's surface closure never resets its projection point count
    (``num_points_in_projection`` is doubled per projection for the whole
    body, ``src/BFLBody.cpp:572,654``), so its cost doubles with every
    closure marker and a circle needing a few dozen of them never finishes
    setting up.  ``reset_projection`` starts every closure from the initial
    20 points instead (a circle the reference can set up may then get
    slightly different closure positions); the default follows the
    reference."""
    if level0.defs.dims != 2:
        raise ValueError("circle_body builds the 2D prefab")
    return _build(level0, prefab_points(level0, centre, radius), reset_projection)


def sphere_body(level0, centre, radius: float, reset_projection: bool = False) -> BflBody:
    """A rigid 3D BFL sphere on level 0 (reference ``CIRCLE_SPHERE BFL`` in
    3D): the Fibonacci prefab, the same labelling and closure, and the 3D
    ``computeQ`` (``src/BFLBody.cpp:244-404``): line-triangle intersections
    of each even direction's link with every triangle of three markers of
    the site's 3x3x3 neighbourhood."""
    if level0.defs.dims != 3:
        raise ValueError("sphere_body builds the 3D prefab")
    return _build(level0, prefab_points(level0, centre, radius), reset_projection)


def _build(lv, points, reset_projection: bool, voxels=None) -> BflBody:
    """Markers at `points` (in order; `voxels`, when given, are their
    primary support voxels, else the voxels enclosing the points), then
    BFLBody::initialise: labels, enforceSurfaceClosure, computeQ, and the
    per-site marker lookup."""
    d = lv.defs
    D = d.dims
    N, M, K, dh = lv.N, lv.M, lv.K, lv.dh
    Q = d.Q
    c = [[int(x) for x in cv] for cv in lattice(D, Q)[0]]
    e = lv.edges if lv.edges is not None else lv.global_edges  # the grid's own edges
    gx0, gy0, gz0 = e[0], e[2], e[4]
    typ = lv.typ.reshape(N, M, K).copy()
    xpos, ypos, zpos = lv.xpos, lv.ypos, lv.zpos

    def voxel(x, y, z):
        return (int(math.floor((x - gx0) / dh)), int(math.floor((y - gy0) / dh)),
                int(math.floor((z - gz0) / dh)) if D == 3 else 0)

    def off_grid(i, j, k):
        return i >= N or i < 0 or j >= M or j < 0 or k >= K or k < 0

    pos, supp = [], []
    voxel_marker = {}  # voxel -> first marker in it (getMarkerData's linear search)

    def add_marker(x, y, z):
        v = voxel(x, y, z)
        if off_grid(*v):
            raise ValueError("BFL marker off the grid")
        voxel_marker.setdefault(v, len(pos))
        pos.append((x, y, z))
        supp.append(v)

    def marker_at(x, y, z):
        v = voxel(x, y, z)
        if off_grid(*v):
            return -1
        return voxel_marker.get(v, -1)

    for n_, p in enumerate(points):
        add_marker(*p)
        if voxels is not None and tuple(voxels[n_]) != supp[-1]:
            v = tuple(voxels[n_])
            if voxel_marker.get(supp[-1]) == len(pos) - 1:
                del voxel_marker[supp[-1]]
            voxel_marker.setdefault(v, len(pos) - 1)
            supp[-1] = v
    for s in supp:
        typ[s] = A.BFL

    # enforceSurfaceClosure: a diagonal eBFL neighbour without an eBFL site
    # connecting the two gets a marker at the mean of the projected points
    # that fall outside eBFL voxels
    npts = 20
    m = 0
    while m < len(pos):
        for di, dj, dk in itertools.product((-1, 1), (-1, 1), (-1, 1) if D == 3 else (0,)):
            ni, nj, nk = supp[m][0] + di, supp[m][1] + dj, supp[m][2] + dk
            if off_grid(ni, nj, nk) or typ[ni, nj, nk] != A.BFL:
                continue
            found = False
            for ic in range(2):
                for jc in range(2):
                    for kc in range(2):
                        is_, js, ks = di - ic * di, dj - jc * dj, dk - kc * dk
                        if (is_, js, ks) == (di, dj, dk) or (is_, js, ks) == (0, 0, 0):
                            continue
                        a, b, e = supp[m][0] + is_, supp[m][1] + js, supp[m][2] + ks
                        if not off_grid(a, b, e) and typ[a, b, e] == A.BFL:
                            found = True
                            break
                    if found:
                        break
                if found:
                    break
            if found:
                continue
            start = pos[m]
            other = pos[marker_at(xpos[ni], ypos[nj], zpos[nk])]
            ln = (other[0] - start[0], other[1] - start[1], other[2] - start[2])
            need, count = False, 0
            av = [0.0, 0.0, 0.0]
            if reset_projection:
                npts = 20
            while not need:
                npts *= 2
                sp = 1.0 / npts
                for p in range(npts + 1):
                    px = start[0] + p * sp * ln[0]
                    py = start[1] + p * sp * ln[1]
                    pz = start[2] + p * sp * ln[2]
                    vi, vj, vk = voxel(px, py, pz)
                    if typ[vi, vj, vk] != A.BFL:
                        if not need:
                            need = True
                            av = [px, py, pz]
                        else:
                            av = [(av[0] * count + px) / (count + 1), (av[1] * count + py) / (count + 1),
                                  (av[2] * count + pz) / (count + 1)]
                        count += 1
                if need:
                    add_marker(av[0], av[1], av[2])
                    typ[supp[-1]] = A.BFL
        m += 1

    nm = len(pos)
    q = np.full(Q * nm, -1.0)
    if D == 2:
        # computeQ (2D): line-line intersections of each link of an eBFL site
        # with the segments to its horizontal/vertical eBFL neighbours
        for i, j in np.argwhere(typ[:, :, 0] == A.BFL).tolist():  # (i, j) order
            store = marker_at(xpos[i], ypos[j], zpos[0])
            combo = []
            for ii in range(i - 1, i + 2):
                for jj in range(j - 1, j + 2):
                    if 0 <= ii < N and 0 <= jj < M and (ii == i or jj == j) and not (ii == i and jj == j):
                        mm = marker_at(xpos[ii], ypos[jj], zpos[0])
                        if mm >= 0:
                            combo.append((store, mm))
            if not combo:
                continue
            q0 = pos[store]
            for first, second in combo:
                qps = pos[second]
                p = (xpos[i], ypos[j], pos[first][2])
                for vel in range(Q - 1):
                    di_ = (i + c[vel][0] + N) % N
                    dj_ = (j + c[vel][1] + M) % M
                    ppr = (xpos[di_], ypos[dj_], pos[first][2])
                    s1x, s1y = ppr[0] - p[0], ppr[1] - p[1]
                    s2x, s2y = qps[0] - q0[0], qps[1] - q0[1]
                    den = -s2x * s1y + s1x * s2y
                    if den == 0.0:
                        continue  # parallel: the reference's s and t are inf or nan
                    s = (-s1y * (p[0] - q0[0]) + s1x * (p[1] - q0[1])) / den
                    t = (s2x * (p[1] - q0[1]) - s2y * (p[0] - q0[0])) / den
                    if s >= 0 and s <= 1 and t >= 0 and t <= 1:
                        ix, iy = p[0] + t * s1x, p[1] + t * s1y
                        wd = _vecnorm((ix - p[0], iy - p[1], p[2] - p[2])) / \
                            _vecnorm((ppr[0] - p[0], ppr[1] - p[1], ppr[2] - p[2]))
                        k = vel + Q * store
                        if q[k] == -1:
                            q[k] = np.finfo(np.float64).max
                        if wd < q[k]:
                            q[k] = wd
    else:
        # computeQ (3D): each even direction's link against every triangle
        # of three markers of the site's 3x3x3 neighbourhood (ids sorted)
        for i, j, k in np.argwhere(typ == A.BFL).tolist():  # (i, j, k) order
            store = marker_at(xpos[i], ypos[j], zpos[k])
            V = []
            for ii in range(i - 1, i + 2):
                for jj in range(j - 1, j + 2):
                    for kk in range(k - 1, k + 2):
                        if 0 <= ii < N and 0 <= jj < M and 0 <= kk < K:
                            mm = marker_at(xpos[ii], ypos[jj], zpos[kk])
                            if mm >= 0:
                                V.append(mm)
            if len(V) < 3:
                continue
            V.sort()
            src = (xpos[i], ypos[j], zpos[k])
            for t0, t1, t2 in itertools.combinations(V, 3):
                o = pos[t0]
                u = (pos[t1][0] - o[0], pos[t1][1] - o[1], pos[t1][2] - o[2])
                v = (pos[t2][0] - o[0], pos[t2][1] - o[1], pos[t2][2] - o[2])
                nrm = (u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0])
                if _vecnorm(nrm) == 0:
                    continue  # degenerate triangle
                uu, uv, vv = _dot(u, u), _dot(u, v), _dot(v, v)
                Dd = uv * uv - uu * vv
                w0 = (src[0] - o[0], src[1] - o[1], src[2] - o[2])
                a = -_dot(nrm, w0)
                for vel in range(0, Q - 1, 2):
                    dst = (xpos[(i + c[vel][0] + N) % N], ypos[(j + c[vel][1] + M) % M],
                           zpos[(k + c[vel][2] + K) % K])
                    dr = (dst[0] - src[0], dst[1] - src[1], dst[2] - src[2])
                    b = _dot(nrm, dr)
                    if abs(b) < 1e-8:  # L_SMALL_NUMBER: parallel or in-plane
                        continue
                    r = a / b
                    if r < 0 or r > 1:
                        continue
                    ip = (src[0] + dr[0] * r, src[1] + dr[1] * r, src[2] + dr[2] * r)
                    w = (ip[0] - o[0], ip[1] - o[1], ip[2] - o[2])
                    wu, wv = _dot(w, u), _dot(w, v)
                    s_ = (uv * wv - vv * wu) / Dd
                    t_ = (uv * wu - uu * wv) / Dd
                    if s_ < 0.0 or s_ > 1.0:
                        continue
                    if t_ < 0.0 or (s_ + t_) > 1.0:
                        continue
                    qd = _vecnorm((ip[0] - src[0], ip[1] - src[1], ip[2] - src[2])) / _vecnorm(dr)
                    kq = vel + Q * store
                    if q[kq] == -1:
                        q[kq] = np.finfo(np.float64).max
                    if qd < q[kq]:
                        q[kq] = qd
    # a site's position lies in its own voxel: the lookup is the first
    # marker of the voxel
    site_marker = np.full(N * M * K, -1, dtype=np.int32)
    for (i, j, k), m in voxel_marker.items():
        site_marker[k + j * K + i * K * M] = m
    return BflBody(typ=typ.reshape(-1), site_marker=site_marker, q=q.reshape(nm, Q), positions=np.array(pos))
