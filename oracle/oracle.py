"""ORACLE — test infrastructure only: loader for the CPU restatement.

Builds ``oracle/_build/liboracle.so`` from ``lbm_oracle.c`` (and the IBM
restatement) with gcc and exposes it through ctypes with the same shape as
the GPU C ABI (create / upload / step / download).  Only tests, the smoke
check and the benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SOURCES = ["lbm_oracle.c"]

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
from luma_gb300 import _abi as A  # noqa: E402


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(ROOT, "include", "luma_gpu.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(map(os.path.getmtime, deps)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", "-std=c11",
           "-o", tmp, *srcs, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.oracle_grid_create.restype = C.c_void_p
        L.oracle_grid_create.argtypes = [C.POINTER(A.GridDesc), C.c_void_p]
        L.oracle_grid_destroy.argtypes = [C.c_void_p]
        L.oracle_upload_state.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4 + [C.c_int]
        L.oracle_download_state.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
        L.oracle_equilibrium.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3
        L.oracle_step.argtypes = [C.c_void_p, C.c_int]
        L.oracle_get_time.argtypes = [C.c_void_p]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_ibm_add_body.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double)]
        L.oracle_ibm_initialise.argtypes = []
        L.oracle_ibm_set_universal.argtypes = [C.c_int]
        L.oracle_ibm_markers.argtypes = [C.c_int, C.POINTER(C.c_double)]
        L.oracle_ibm_supports.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_int]
        L.oracle_ibm_reset.argtypes = []
        L.oracle_ibm_add_filament.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.c_double, C.c_double,
                                              C.c_double, C.c_double, C.c_int, C.c_int, C.c_double,
                                              C.c_double, C.c_double, C.c_double]
        L.oracle_fem_state.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.oracle_momex_force.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_bfl_set.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double)]
        L.oracle_bfl_forces.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_download_fnew.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_download_time_averages.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 3
        L.oracle_kbc_gamma.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.oracle_lu_solve_rowmajor.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_lattice.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]
        L.oracle_delta.restype = C.c_double
        L.oracle_delta.argtypes = [C.c_double, C.c_double]
        L.oracle_guo.argtypes = [C.c_int, C.c_int, C.c_double] + [C.POINTER(C.c_double)] * 3
        _lib = L
    return _lib


def lattice(Q: int) -> dict:
    """The oracle's lattice tables: c (Q, 3), w (Q,), opp (Q,), refl (3, Q)."""
    c = np.zeros(3 * Q, dtype=np.int32)
    w = np.zeros(Q)
    opp = np.zeros(Q, dtype=np.int32)
    refl = np.zeros(3 * Q, dtype=np.int32)
    ip = C.POINTER(C.c_int)
    if lib().oracle_lattice(Q, c.ctypes.data_as(ip), A.dptr(w), opp.ctypes.data_as(ip), refl.ctypes.data_as(ip)):
        raise RuntimeError(lib().oracle_last_error().decode())
    return {"c": c.reshape(Q, 3), "w": w, "opp": opp, "refl": refl.reshape(3, Q)}


def delta(r: float, dilation: float = 1.0) -> float:
    return lib().oracle_delta(float(r), float(dilation))


def guo(Q: int, dims: int, omega: float, u, F) -> np.ndarray:
    """Guo forcing terms F_i of one site with velocity u and force F."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    out = np.zeros(Q)
    lib().oracle_guo(Q, dims, float(omega), A.dptr(u), A.dptr(F), A.dptr(out))
    return out


def lu_solve(M: np.ndarray, b: np.ndarray) -> np.ndarray:
    """The oracle's dense partial-pivot LU solve of M x = b (M row-major)."""
    a = np.array(M, dtype=np.float64, order="C", copy=True)
    x = np.array(b, dtype=np.float64, copy=True)
    lib().oracle_lu_solve_rowmajor(int(a.shape[0]), A.dptr(a), A.dptr(x))
    return x


class OracleGrid:
    """One grid of the CPU restatement (reference AoS layout on the host)."""

    def __init__(self, desc: "A.GridDesc", parent: "OracleGrid | None" = None):
        self.desc = desc
        self.L = lib()
        self.h = self.L.oracle_grid_create(C.byref(desc), parent.h if parent else None)
        if not self.h:
            raise RuntimeError(self.L.oracle_last_error().decode())
        self.n = desc.N * desc.M * desc.K
        self.children: list[OracleGrid] = []
        self.parent = parent
        if parent is not None:
            parent.children.append(self)

    def close(self):
        if self.h and self.parent is None:
            self.L.oracle_grid_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, f=None, u=None, rho=None, force=None, t: int = 0):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (f, u, rho, force)]
        self.L.oracle_upload_state(self.h, *[A.dptr(a) for a in arrs], t)

    def download(self):
        d = self.desc
        f = np.empty(self.n * d.Q)
        u = np.empty(self.n * d.dims)
        rho = np.empty(self.n)
        force = np.empty(self.n * d.dims)
        self.L.oracle_download_state(self.h, A.dptr(f), A.dptr(u), A.dptr(rho), A.dptr(force))
        return {"f": f, "u": u, "rho": rho, "force": force}

    def momex_force(self) -> np.ndarray:
        """Momentum-exchange force of the solid sites (computeLiftDrag)."""
        out = np.zeros(3)
        self.L.oracle_momex_force(self.h, A.dptr(out))
        return out

    def kbc_gamma(self) -> np.ndarray:
        """The KBC stabiliser gamma of each site's latest collision (NaN
        where none ran)."""
        out = np.empty(self.n)
        if self.L.oracle_kbc_gamma(self.h, A.dptr(out)):
            raise RuntimeError(self.L.oracle_last_error().decode())
        return out

    def time_averages(self) -> dict:
        """Running means (reference layout): rho (n), u (n*D), uu (n*(3D-3))."""
        d = self.desc
        n = d.N * d.M * d.K
        out = {"rho": np.zeros(n), "u": np.zeros(n * d.dims), "uu": np.zeros(n * (3 * d.dims - 3))}
        if self.L.oracle_download_time_averages(self.h, A.dptr(out["rho"]), A.dptr(out["u"]), A.dptr(out["uu"])):
            raise RuntimeError(self.L.oracle_last_error().decode())
        return out

    def fnew(self) -> np.ndarray:
        """GridObj::fNew between steps (the state before the latest step)."""
        out = np.zeros(self.desc.N * self.desc.M * self.desc.K * self.desc.Q)
        self.L.oracle_download_fnew(self.h, A.dptr(out))
        return out

    def bfl_set(self, site_marker, q) -> None:
        """BFL body 0: per-site marker of the site's voxel (-1 for none) and
        the (nm, Q) link distances (-1: no wall on the link)."""
        sm = np.ascontiguousarray(site_marker, dtype=np.int32)
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._bfl_nm = int(q.shape[0])
        if self.L.oracle_bfl_set(self.h, sm.ctypes.data_as(C.POINTER(C.c_int)), self._bfl_nm, A.dptr(q)):
            raise RuntimeError(self.L.oracle_last_error().decode())

    def bfl_forces(self) -> np.ndarray:
        """(nm, 3) momentum-exchange force per BFL marker of the latest step."""
        out = np.zeros((self._bfl_nm, 3))
        if self.L.oracle_bfl_forces(self.h, A.dptr(out)):
            raise RuntimeError(self.L.oracle_last_error().decode())
        return out

    def equilibrium(self, u, rho):
        d = self.desc
        u = np.ascontiguousarray(u, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        f = np.empty(self.n * d.Q)
        self.L.oracle_equilibrium(self.h, A.dptr(u), A.dptr(rho), A.dptr(f))
        return f

    def step(self, nsteps: int = 1):
        if self.L.oracle_step(self.h, nsteps) != 0:
            raise RuntimeError(self.L.oracle_last_error().decode())

    @property
    def t(self) -> int:
        return self.L.oracle_get_time(self.h)


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(n)


class OracleIBM:
    """Rigid IB bodies of the oracle (one process-wide set)."""

    def __init__(self):
        self.L = lib()
        self.L.oracle_ibm_reset()
        self.nm = []

    def add_body(self, grid: OracleGrid, positions) -> int:
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        ib = self.L.oracle_ibm_add_body(grid.h, pos.shape[0], A.dptr(pos))
        self.nm.append(pos.shape[0])
        return ib

    def initialise(self, universal: bool = False):
        """ibm_initialise; `universal` = L_UNIVERSAL_EPSILON_CALC."""
        self.L.oracle_ibm_set_universal(1 if universal else 0)
        if self.L.oracle_ibm_initialise() != 0:
            raise RuntimeError(self.L.oracle_last_error().decode())

    def markers(self, ib: int) -> np.ndarray:
        out = np.empty((self.nm[ib], 9))
        self.L.oracle_ibm_markers(ib, A.dptr(out))
        return out

    def supports(self, ib: int) -> np.ndarray:
        n = self.L.oracle_ibm_supports(ib, None, 0)
        out = np.empty((n, 5))
        self.L.oracle_ibm_supports(ib, A.dptr(out), n)
        return out

    def add_filament(self, grid: OracleGrid, start, length, height, depth, angle_v, nel, clamped, density, E,
                     dm, fsi_vel_scale) -> int:
        st = np.ascontiguousarray(start, dtype=np.float64)
        ib = self.L.oracle_ibm_add_filament(grid.h, A.dptr(st), length, height, depth, angle_v, nel,
                                            int(clamped), density, E, dm, fsi_vel_scale)
        if ib < 0:
            raise RuntimeError(self.L.oracle_last_error().decode())
        import math
        self.nm.append(int(math.floor(length / grid.desc.dh)) + 1)
        return ib

    def fem_state(self, k: int):
        nd = C.c_int()
        self.L.oracle_fem_state(k, None, C.byref(nd), None, None)
        U = np.empty(nd.value)
        it = C.c_int()
        res = C.c_double()
        self.L.oracle_fem_state(k, A.dptr(U), C.byref(nd), C.byref(it), C.byref(res))
        return U, it.value, res.value
