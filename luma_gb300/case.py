"""Host-side case set-up: the definitions-driven initialisation of a level-0 grid.

Mirrors the reference's compile-time configuration (LUMA ``inc/definitions.h``)
and the L0 initialisation that consumes it, producing exactly the inputs the
time step reads:

* global edges ``dh * L_N`` etc. (``src/GridManager.cpp:45-51``);
* site positions ``linspace(dh/2, edge - dh/2, n)`` (``src/GridObj_init_grids.cpp:237-245``,
  ``inc/GridUtils.h:289-308``);
* wall labels with the reference's precedence (``LBM_initBoundLab``,
  ``src/GridObj_init_grids.cpp:983-1097``; ``LBM_setBCPrecedence`` :1372-1377);
* the inlet profile (``_LBM_initSetInletProfile`` :1322-1360);
* initial u, rho (``LBM_initVelocity``/``LBM_initRho`` :37-152) and
  ``nu``/``omega`` (:336-344);
* the Guo force field at t=0 under gravity (:284-291).

Arithmetic follows the reference's expression order so the values are
bit-identical to those the reference computes.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

CS = 1.0 / math.sqrt(3.0)


@dataclass
class Definitions:
    """The subset of ``definitions.h`` switches that shape the time step."""

    dims: int = 2
    resolution: int = 100          # L_RESOLUTION
    timestep: float = 0.0001       # L_TIMESTEP
    bx: float = 1.0                # L_BX
    by: float = 1.0                # L_BY
    bz: float = 1.0                # L_BZ
    re: float | None = 100.0       # L_RE
    nu: float | None = None        # L_NU (overrides L_RE when set)
    ux0: float = 0.0               # L_UX0
    uy0: float = 0.0               # L_UY0
    uz0: float = 0.0               # L_UZ0
    rho_in: float = 1.0            # L_RHOIN
    parabolic_inlet: bool = False  # L_PARABOLIC_INLET
    inlet_profile: str | None = None  # L_USE_INLET_PROFILE: text of input/inlet_profile.in
    no_flow: bool = True           # L_NO_FLOW
    velocity_ramp: float = 0.0     # L_VELOCITY_RAMP (0 = undefined)
    reynolds_ramp: float = 0.0     # L_REYNOLDS_RAMP (0 = undefined)
    time_averages: bool = False    # L_COMPUTE_TIME_AVERAGED_QUANTITIES
    regularised: bool = False      # L_REGULARISED_BOUNDARIES
    kbc: bool = False              # L_USE_KBC_COLLISION
    smagorinsky: bool = False      # L_USE_BGKSMAG
    csmag: float = 0.3             # L_CSMAG
    ibm: bool = False              # L_IBM_ON
    universal_epsilon: bool = False  # L_UNIVERSAL_EPSILON_CALC
    gravity: bool = False          # L_GRAVITY_ON
    gravity_force: float = 0.0     # L_GRAVITY_FORCE
    gravity_dir: int = 0           # L_GRAVITY_DIRECTION
    pressure_delta: float = 0.0    # L_PRESSURE_DELTA
    physical_rho: float = 1000.0   # L_PHYSICAL_RHO
    # L_WALL_LEFT, RIGHT, BOTTOM, TOP, FRONT, BACK
    walls: tuple = (A.FLUID,) * 6
    # L_WALL_THICKNESS_* in coarse cells
    wall_cells: tuple = (1.0,) * 6

    @property
    def Q(self) -> int:
        if self.dims == 2:
            return 9
        return 27 if self.kbc else 19

    def sizes(self) -> tuple[int, int, int]:
        n = int(self.bx * self.resolution)
        m = int(self.by * self.resolution)
        k = int(self.bz * self.resolution) if self.dims == 3 else 1
        return n, m, k


@dataclass
class Level0:
    defs: Definitions
    N: int
    M: int
    K: int
    dh: float
    dt: float
    nu: float
    omega: float
    gravity: float
    global_edges: np.ndarray
    wall_thickness: np.ndarray
    xpos: np.ndarray
    ypos: np.ndarray
    zpos: np.ndarray
    typ: np.ndarray
    ux_in: np.ndarray
    uy_in: np.ndarray
    uz_in: np.ndarray
    u: np.ndarray
    rho: np.ndarray
    force_xyz: np.ndarray = field(default=None)
    level: int = 0
    region: int = 0
    coarse_lims: tuple = (0, 0, 0, 0, 0, 0)
    refinement_ratio: float = 1.0
    edges: tuple = None          # this grid's global edges (x/y/z min,max)

    @property
    def ncell(self) -> int:
        return self.N * self.M * self.K

    def flags(self, fix_macro3d: bool = False, fix_kbc: bool = False) -> int:
        d = self.defs
        fl = 0
        if d.regularised:
            fl |= A.FLAG_REGULARISED
        if d.ibm:
            fl |= A.FLAG_IBM
        if d.gravity:
            fl |= A.FLAG_GRAVITY
        if d.time_averages:
            fl |= A.FLAG_TIME_AVERAGES
        if d.universal_epsilon:
            fl |= A.FLAG_UNIVERSAL_EPSILON
        if fix_macro3d:
            fl |= A.FLAG_FIX_MACRO3D
        if fix_kbc:
            fl |= A.FLAG_FIX_KBC
        return fl

    def desc(self, precision: int = A.PREC_FP64, fix_macro3d: bool = False,
             fix_kbc: bool = False) -> "A.GridDesc":
        """A level-0 ``luma_grid_desc``; keeps the arrays it points to alive."""
        d = self.defs
        g = A.GridDesc()
        g.abi_version = A.ABI_VERSION
        g.level, g.region = self.level, self.region
        g.dims, g.Q = d.dims, d.Q
        g.N, g.M, g.K = self.N, self.M, self.K
        g.precision = precision
        g.collision = A.COLL_KBC if d.kbc else (A.COLL_BGK_SMAG if d.smagorinsky else A.COLL_BGK)
        g.flags = self.flags(fix_macro3d, fix_kbc)
        g.omega, g.dt, g.dh = self.omega, self.dt, self.dh
        g.refinement_ratio = self.refinement_ratio
        for q in range(6):
            g.coarse_lims[q] = int(self.coarse_lims[q])
        g.rho_in = d.rho_in
        g.velocity_ramp = d.velocity_ramp
        g.reynolds_ramp = d.reynolds_ramp
        g.re = float(d.re) if d.re is not None else 0.0
        g.pressure_delta = pd2dlbm(d.pressure_delta, self.dh, self.dt, self.dm)
        g.gravity = self.gravity
        g.gravity_dir = d.gravity_dir
        g.csmag = d.csmag
        for i in range(6):
            g.global_edges[i] = float(self.global_edges[i])
            g.wall_thickness[i] = float(self.wall_thickness[i])
        keep = (np.ascontiguousarray(self.typ, dtype=np.int32),
                np.ascontiguousarray(self.xpos), np.ascontiguousarray(self.ypos),
                np.ascontiguousarray(self.zpos), np.ascontiguousarray(self.ux_in),
                np.ascontiguousarray(self.uy_in), np.ascontiguousarray(self.uz_in))
        g.lattyp = A.iptr(keep[0])
        g.xpos, g.ypos, g.zpos = A.dptr(keep[1]), A.dptr(keep[2]), A.dptr(keep[3])
        g.ux_in, g.uy_in, g.uz_in = A.dptr(keep[4]), A.dptr(keep[5]), A.dptr(keep[6])
        g._keep = keep
        return g

    @property
    def dm(self) -> float:
        return (self.defs.physical_rho / self.defs.rho_in) * self.dh * self.dh * self.dh


GridLevel = Level0


def pd2dlbm(p: float, dh: float, dt: float, dm: float) -> float:
    """GridUnits::pd2dlbm (inc/GridUnits.h:171-174)."""
    return (p * dh * (dt * dt) / dm) / (CS * CS)


def linspace(lo: float, hi: float, n: int) -> np.ndarray:
    """GridUtils::linspace (inc/GridUtils.h:289-308): lo + spacing*i."""
    n = max(n, 2)
    spacing = (hi - lo) / float(n - 1)
    return np.array([lo + spacing * i for i in range(n)], dtype=np.float64)


def ramp_coefficient(defs: Definitions, t: float) -> float:
    """GridUtils::getVelocityRampCoefficient (src/GridUtils.cpp:1808-1816)."""
    if defs.velocity_ramp > 0 and t <= defs.velocity_ramp:
        return (1.0 - math.cos(math.pi * t / defs.velocity_ramp)) / 2.0
    return 1.0


def _precedence(cur: int, want: int) -> int:
    """LBM_setBCPrecedence (src/GridObj_init_grids.cpp:1372-1377)."""
    if cur == A.SOLID or want == A.SOLID:
        return A.SOLID
    if cur == A.VELOCITY:
        return A.VELOCITY
    return want


def _precedence_array(cur: np.ndarray, want: int) -> np.ndarray:
    """_precedence over an array of current labels."""
    out = np.full(cur.shape, want, dtype=cur.dtype)
    out[cur == A.VELOCITY] = A.VELOCITY
    out[cur == A.SOLID] = A.SOLID
    if want == A.SOLID:
        out[...] = A.SOLID
    return out


def _initial_velocity(defs: Definitions, typ: np.ndarray, prof: np.ndarray) -> np.ndarray:
    """LBM_initVelocity (src/GridObj_init_grids.cpp:37-152): the inlet
    profile of each row (velocity sites only under L_NO_FLOW), zero at solid
    sites.  typ has shape (N, M, K), prof (M, D)."""
    N, M, K = typ.shape
    D = prof.shape[1]
    u = np.zeros((N, M, K, D))
    use = np.ones(typ.shape, dtype=bool) if not defs.no_flow else (typ == A.VELOCITY)
    prof_b = np.broadcast_to(prof[None, :, None, :], (N, M, K, D))
    u[use] = prof_b[use]
    u[typ == A.SOLID] = 0.0
    return u


_NUMBER = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)?(?:[eE][+-]?\d*)?")


class _StreamReader:
    """Formatted extraction of doubles from one std::istringstream that is
    refilled line by line with str() + seekg(0), as
    GridUtils::readVelocityFromFile does: seekg clears only end-of-file, so
    once an extraction has failed every later one fails too and leaves the
    variable as it was; an extraction that finds no whitespace-delimited
    remainder fails without touching the variable; one that finds
    characters that do not form a number stores 0 and fails."""

    def __init__(self):
        self.failed = False
        self.line = ""
        self.pos = 0
        self.tmp = None

    def reset(self, line: str) -> None:
        self.line, self.pos = line, 0

    def extract(self) -> float | None:
        if self.failed:
            return self.tmp
        while self.pos < len(self.line) and self.line[self.pos].isspace():
            self.pos += 1
        if self.pos >= len(self.line):
            self.failed = True
            return self.tmp
        m = _NUMBER.match(self.line, self.pos)
        text = m.group(0)
        mant = re.match(r"[+-]?(\d+\.?\d*|\.\d+)", text)
        exp = text[mant.end():] if mant else ""
        if not mant or (exp and not re.fullmatch(r"[eE][+-]?\d+", exp)):
            self.pos = m.end()
            self.failed = True
            self.tmp = 0.0
            return self.tmp
        self.pos = m.end()
        self.tmp = float(text)
        return self.tmp


def initial_velocity_from_file(text: str, l0: "Level0") -> np.ndarray:
    """Level-0 velocity under L_INIT_VELOCITY_FROM_FILE (LBM_initVelocity,
    src/GridObj_init_grids.cpp:42-78, with GridUtils::readVelocityFromFile,
    src/GridUtils.cpp:1467-1524) from the text of
    ``input/initial_velocity.in``: one point "x y z ux uy uz" per line in
    dimensionless units, read with the stream semantics of ``_StreamReader``
    (the empty line after a final newline adds a point repeating the last
    value read); the first N*M*K points in file order are applied, each to
    the site enclosing its position (points off the grid are skipped, later
    points overwrite earlier ones), as u * dt / dh; every other site keeps
    u = 0 (no profile, no zeroing of solid sites).  Fewer points than sites
    raise ValueError, as the reference stops there."""
    rd = _StreamReader()
    cols = [[] for _ in range(6)]
    lines = text.split("\n")
    for line in lines:
        rd.reset(line)
        for c in cols:
            c.append(rd.extract())
    n = l0.N * l0.M * l0.K
    if len(cols[0]) < n:
        raise ValueError(f"initial velocity file has {len(cols[0])} points for {n} sites")
    if any(v is None for c in cols for v in c[:n]):
        raise ValueError("initial velocity file: a value read before any number (uninitialised in the reference)")
    D = l0.defs.dims
    E = l0.global_edges
    u = np.zeros((l0.N, l0.M, l0.K, D))
    for p in range(n):
        x, y, z = cols[0][p], cols[1][p], cols[2][p]
        if not (E[0] <= x < E[1] and E[2] <= y < E[3] and (D != 3 or E[4] <= z < E[5])):
            continue
        i = int(math.floor((x - E[0]) / l0.dh))
        j = int(math.floor((y - E[2]) / l0.dh))
        k = int(math.floor((z - E[4]) / l0.dh)) if D == 3 else 0
        if not (0 <= i < l0.N and 0 <= j < l0.M and 0 <= k < l0.K):
            continue
        for d in range(D):
            u[i, j, k, d] = (cols[3 + d][p] * l0.dt) / l0.dh
    return u.reshape(-1)


def inlet_profile_from_file(text: str, ypos: np.ndarray) -> tuple:
    """L_USE_INLET_PROFILE (_LBM_initGetInletProfileFromFile,
    src/GridObj_init_grids.cpp:1234-1314): the points of
    ``input/inlet_profile.in`` ("x y z ux uy uz" lines, read as
    ``initial_velocity_from_file`` reads, so a final newline appends a point
    whose every value is the last one read), taken in file order for each
    site row y: below the first point, linear extrapolation from the first
    two; above the last, from the last two; between two consecutive points,
    linear interpolation; on a point, its values.  The values are used as
    they are (lattice units); a row no rule reaches keeps 0."""
    rd = _StreamReader()
    cols = [[] for _ in range(6)]
    for line in text.split("\n"):
        rd.reset(line)
        for c in cols:
            c.append(rd.extract())
    if any(v is None for c in cols for v in c):
        raise ValueError("inlet profile file: a value read before any number (uninitialised in the reference)")
    yb, ub = cols[1], cols[3:6]
    if len(yb) < 2:
        raise ValueError("inlet profile file: the rules need at least two points")
    M = ypos.size
    out = [np.zeros(M), np.zeros(M), np.zeros(M)]
    last = len(yb) - 1
    for j in range(M):
        y = float(ypos[j])
        for i in range(len(yb)):
            if i == 0 and yb[i] > y:
                for o, u in zip(out, ub):
                    o[j] = -(u[i + 1] - u[i]) + u[i]
                break
            if i == last and yb[i] < y:
                for o, u in zip(out, ub):
                    o[j] = (u[i] - u[i - 1]) + u[i]
                break
            if yb[i] < y and yb[i + 1] > y:
                for o, u in zip(out, ub):
                    o[j] = ((u[i + 1] - u[i]) / (yb[i + 1] - yb[i])) * (y - yb[i]) + u[i]
                break
            if yb[i] == y:
                for o, u in zip(out, ub):
                    o[j] = u[i]
                break
    return tuple(out)


def build_level0(defs: Definitions) -> Level0:
    N, M, K = defs.sizes()
    dh = 1.0 / float(defs.resolution)
    dt = defs.timestep
    edges = np.array([0.0, dh * N, 0.0, dh * M, 0.0, dh * K if defs.dims == 3 else 0.0])
    wt = np.array([c * dh for c in defs.wall_cells], dtype=np.float64)
    xpos = linspace(dh / 2.0, edges[1] - dh / 2.0, N)
    ypos = linspace(dh / 2.0, edges[3] - dh / 2.0, M)
    zpos = linspace(dh / 2.0, edges[5] - dh / 2.0, K) if defs.dims == 3 else np.zeros(1)

    typ = np.full((N, M, K), A.FLUID, dtype=np.int32)
    left, right, bottom, top, front, back = defs.walls

    def label(sel, want):
        typ[sel] = _precedence_array(typ[sel], want)

    for i in range(N):
        if xpos[i] <= wt[0]:
            label((slice(i, i + 1), slice(None), slice(None)), left)
    for i in range(N):
        if xpos[i] >= edges[1] - wt[1]:
            label((slice(i, i + 1), slice(None), slice(None)), right)
    if defs.dims == 3:
        for k in range(K):
            if zpos[k] <= wt[4]:
                label((slice(None), slice(None), slice(k, k + 1)), front)
        for k in range(K):
            if zpos[k] >= edges[5] - wt[5]:
                label((slice(None), slice(None), slice(k, k + 1)), back)
    for j in range(M):
        if ypos[j] <= wt[2]:
            label((slice(None), slice(j, j + 1), slice(None)), bottom)
    for j in range(M):
        if ypos[j] >= edges[3] - wt[3]:
            label((slice(None), slice(j, j + 1), slice(None)), top)

    # Inlet profile.
    if defs.inlet_profile is not None:
        ux_in, uy_in, uz_in = inlet_profile_from_file(defs.inlet_profile, ypos)
    elif defs.parabolic_inlet:
        b = edges[3] - wt[3]
        p = (b + wt[2]) / 2.0
        q = b - p
        umax = (1.5 * defs.ux0 * dt) / dh
        ux_in = np.array([umax * (1.0 - math.pow((ypos[j] - p) / q, 2.0)) for j in range(M)])
        uy_in = np.zeros(M)
        uz_in = np.zeros(M)
    else:
        ux_in = np.full(M, (defs.ux0 * dt) / dh)
        uy_in = np.full(M, (defs.uy0 * dt) / dh)
        uz_in = np.full(M, (defs.uz0 * dt) / dh)

    # Initial velocity and density.
    D = defs.dims
    rc = ramp_coefficient(defs, 0.0)
    prof = np.stack([ux_in * rc, uy_in * rc, uz_in * rc], axis=1)[:, :D]
    u = _initial_velocity(defs, typ, prof)
    rho = np.full((N, M, K), float(defs.rho_in))

    nu_d = defs.nu if defs.nu is not None else 1.0 / float(defs.re)
    nu = (nu_d * dt) / (dh * dh)
    omega = 1.0 / ((nu / (CS * CS)) + 0.5)
    gravity = (defs.gravity_force * (dt * dt)) / dh
    force = np.zeros((N, M, K, D))
    if defs.gravity:
        force[..., defs.gravity_dir] = rho * gravity * 1.0
    return Level0(defs=defs, N=N, M=M, K=K, dh=dh, dt=dt, nu=nu, omega=omega, gravity=gravity,
                  global_edges=edges, wall_thickness=wt, xpos=xpos, ypos=ypos, zpos=zpos,
                  typ=typ.reshape(-1), ux_in=ux_in, uy_in=uy_in, uz_in=uz_in,
                  u=u.reshape(-1), rho=rho.reshape(-1), force_xyz=force.reshape(-1),
                  edges=tuple(edges))


def _inlet_profile(defs: Definitions, ypos: np.ndarray, dt: float, dh: float, edges0) -> tuple:
    """_LBM_initSetInletProfile (src/GridObj_init_grids.cpp:1322-1360) on any grid."""
    M = ypos.size
    if defs.inlet_profile is not None:
        return inlet_profile_from_file(defs.inlet_profile, ypos)
    if defs.parabolic_inlet:
        wt_top = defs.wall_cells[3] / float(defs.resolution)
        wt_bot = defs.wall_cells[2] / float(defs.resolution)
        b = edges0[3] - wt_top
        p = (b + wt_bot) / 2.0
        q = b - p
        umax = (1.5 * defs.ux0 * dt) / dh
        return (np.array([umax * (1.0 - math.pow((ypos[j] - p) / q, 2.0)) for j in range(M)]),
                np.zeros(M), np.zeros(M))
    return (np.full(M, (defs.ux0 * dt) / dh), np.full(M, (defs.uy0 * dt) / dh),
            np.full(M, (defs.uz0 * dt) / dh))


def cround(v: float) -> float:
    """std::round: halves away from zero (Python's round takes them to the
    even neighbour)."""
    r = math.floor(abs(v))
    if abs(v) - r >= 0.5:
        r += 1
    return math.copysign(r, v)


def build_subgrid(parent: "Level0", start: tuple, end: tuple, region: int = 0,
                  coarse_dh_for_edges: float | None = None) -> "Level0":
    """One embedded refined grid (factor 2) inside `parent`, mirroring the
    reference's serial set-up: GridManager edges rounded to the grid spacing
    (src/GridManager.cpp:85-90), coarse limits from the enclosing parent
    voxels of the first/last fine voxel centres (LBM_initGridToGridMappings,
    src/GridObj_init_grids.cpp:547-888; GridUtils::getEnclosingVoxel,
    src/GridUtils.cpp:1625-1719), fine positions (LBM_initPositionVector,
    :902-975), parent relabelling to transition-to-finer / refined and child
    labels from the parent (LBM_initRefinedLab, :1106-1224), and the fine
    relaxation frequency (:527).  `parent.typ` is relabelled in place."""
    defs = parent.defs
    D = defs.dims
    dh_p = parent.dh
    dh = dh_p / 2.0
    dt = parent.dt / 2.0
    rdh = coarse_dh_for_edges if coarse_dh_for_edges is not None else dh_p
    edges = []
    for a_ in range(3):
        if a_ == 2 and D == 2:
            edges += [0.0, 0.0]
            continue
        lo = cround(start[a_] / rdh) * rdh
        hi = cround(end[a_] / rdh) * rdh
        edges += [lo, hi]
    pstart = [parent.edges[0], parent.edges[2], parent.edges[4]]
    ppos = [parent.xpos, parent.ypos, parent.zpos]
    lims = [0, 0, 0, 0, 0, 0]
    sizes = [1, 1, 1]
    pos = [None, None, np.zeros(1)]
    for a_ in range(D):
        lo = int(math.floor(((edges[2 * a_] + dh / 2.0) - pstart[a_]) / dh_p))
        hi = int(math.floor(((edges[2 * a_ + 1] - dh / 2.0) - pstart[a_]) / dh_p))
        lims[2 * a_], lims[2 * a_ + 1] = lo, hi
        sizes[a_] = int((hi - lo + .5) * 2) + 1
        p0 = ppos[a_][lo] - dh / 2.0
        arr = [p0]
        while len(arr) < sizes[a_]:
            arr.append(arr[-1] + dh)
        pos[a_] = np.array(arr)
    N, M, K = sizes
    # Parent relabelling.
    Np, Mp, Kp = parent.N, parent.M, parent.K
    ptyp = parent.typ.reshape(Np, Mp, Kp)
    xp, yp, zp = np.asarray(parent.xpos), np.asarray(parent.ypos), np.asarray(parent.zpos)
    inx = (xp > edges[0]) & (xp < edges[1])
    iny = (yp > edges[2]) & (yp < edges[3])
    inz = ((zp > edges[4]) & (zp < edges[5])) if D == 3 else np.ones(Kp, dtype=bool)
    tlx = ((xp > edges[0]) & (xp < edges[0] + dh_p)) | ((xp < edges[1]) & (xp > edges[1] - dh_p))
    tly = ((yp > edges[2]) & (yp < edges[2] + dh_p)) | ((yp < edges[3]) & (yp > edges[3] - dh_p))
    tlz = (((zp > edges[4]) & (zp < edges[4] + dh_p)) | ((zp < edges[5]) & (zp > edges[5] - dh_p))) if D == 3 \
        else np.zeros(Kp, dtype=bool)
    inside = inx[:, None, None] & iny[None, :, None] & inz[None, None, :]
    tl = tlx[:, None, None] | tly[None, :, None] | tlz[None, None, :]
    fluid = ptyp == A.FLUID
    ptyp[inside & tl & fluid] = A.TL_TO_FINER
    ptyp[inside & ~tl & fluid] = A.REFINED
    parent.typ = ptyp.reshape(-1)
    # Child labels.
    pi = np.arange(N) // 2 + lims[0]
    pj = np.arange(M) // 2 + lims[2]
    pk = (np.arange(K) // 2 + lims[4]) if D == 3 else np.zeros(K, dtype=np.int64)
    pl = ptyp[pi[:, None, None], pj[None, :, None], pk[None, None, :]]
    typ = np.where(pl == A.TL_TO_FINER, A.TL_TO_COARSER, np.where(pl == A.REFINED, A.FLUID, pl)).astype(np.int32)
    ux_in, uy_in, uz_in = _inlet_profile(defs, pos[1], dt, dh, parent_root_edges(parent))
    rc = ramp_coefficient(defs, 0.0)
    prof = np.stack([ux_in * rc, uy_in * rc, uz_in * rc], axis=1)[:, :D]
    u = _initial_velocity(defs, typ, prof)
    rho = np.full((N, M, K), float(defs.rho_in))
    omega = 1.0 / (((1.0 / parent.omega - 0.5) * 2.0) + 0.5)
    level = parent.level + 1
    rr = 1.0 / (2 ** level)
    force = np.zeros((N, M, K, D))
    if defs.gravity:
        force[..., defs.gravity_dir] = rho * parent.gravity * rr
    return Level0(defs=defs, N=N, M=M, K=K, dh=dh, dt=dt, nu=parent.nu, omega=omega, gravity=parent.gravity,
                  global_edges=parent.global_edges, wall_thickness=parent.wall_thickness,
                  xpos=pos[0], ypos=pos[1], zpos=pos[2], typ=typ.reshape(-1), ux_in=ux_in, uy_in=uy_in,
                  uz_in=uz_in, u=u.reshape(-1), rho=rho.reshape(-1), force_xyz=force.reshape(-1),
                  level=level, region=region, coarse_lims=tuple(lims), refinement_ratio=rr, edges=tuple(edges))


def parent_root_edges(g: "Level0"):
    """Global edges of level 0 (every grid keeps them in global_edges)."""
    return g.global_edges


# ---- lattice tables (src/stdafx.cpp:29-153) used by host-side helpers ----

def lattice(dims: int, Q: int):
    """Velocity set ``c`` (Q x 3 ints) and weights ``w`` in the reference's order."""
    if (dims, Q) == (2, 9):
        c = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (1, 1, 0), (-1, -1, 0), (1, -1, 0),
             (-1, 1, 0), (0, 0, 0)]
        w = [1 / 9] * 4 + [1 / 36] * 4 + [4 / 9]
    elif (dims, Q) == (3, 19):
        c = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0),
             (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1),
             (1, 0, 1), (-1, 0, -1), (-1, 0, 1), (1, 0, -1), (0, 0, 0)]
        w = [1 / 18] * 6 + [1 / 36] * 12 + [1 / 3]
    elif (dims, Q) == (3, 27):
        c = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (0, 1, 1),
             (0, -1, -1), (0, 1, -1), (0, -1, 1), (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
             (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 1, 1), (-1, -1, -1), (-1, -1, 1),
             (1, 1, -1), (-1, 1, 1), (1, -1, -1), (1, -1, 1), (-1, 1, -1), (0, 0, 0)]
        w = [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8 + [8 / 27]
    else:
        raise ValueError(f"no lattice D{dims}Q{Q}")
    return np.array(c, dtype=np.int64), np.array(w, dtype=np.float64)


def equilibrium(dims: int, Q: int, rho: np.ndarray, u: np.ndarray) -> np.ndarray:
    """Vectorised _LBM_equilibrium_opt (src/GridObj_ops_lbm_optimised.cpp:674-705).

    ``rho`` has shape (n,), ``u`` shape (n, dims); returns (n, Q) in the
    reference's expression order (bit-identical for IEEE double)."""
    c, w = lattice(dims, Q)
    cs2 = CS * CS
    u = u.reshape(-1, dims)
    out = np.empty((u.shape[0], Q))
    for v in range(Q):
        cv = c[v]
        if dims == 3:
            A_ = (cv[0] * u[:, 0]) + (cv[1] * u[:, 1]) + (cv[2] * u[:, 2])
            B_ = ((cv[0] * cv[0] - cs2) * (u[:, 0] * u[:, 0]) + (cv[1] * cv[1] - cs2) * (u[:, 1] * u[:, 1])
                  + (cv[2] * cv[2] - cs2) * (u[:, 2] * u[:, 2])
                  + float(2 * cv[0] * cv[1]) * u[:, 0] * u[:, 1]
                  + float(2 * cv[0] * cv[2]) * u[:, 0] * u[:, 2]
                  + float(2 * cv[1] * cv[2]) * u[:, 1] * u[:, 2])
        else:
            A_ = (cv[0] * u[:, 0]) + (cv[1] * u[:, 1])
            B_ = ((cv[0] * cv[0] - cs2) * (u[:, 0] * u[:, 0]) + (cv[1] * cv[1] - cs2) * (u[:, 1] * u[:, 1])
                  + float(2 * cv[0] * cv[1]) * u[:, 0] * u[:, 1])
        out[:, v] = rho * w[v] * (1.0 + (A_ / cs2) + (B_ / (2.0 * cs2 * cs2)))
    return out
