"""ctypes binding of the GB300 C ABI (``include/luma_gpu.h``).

``GpuGrid`` mirrors one GridObj of the reference's hierarchy on the device:
create from a ``luma_grid_desc``, upload/download state in the reference's
host layout, and ``step`` = ``GridObj::LBM_multi_opt`` (LUMA
src/GridObj_ops_lbm_optimised.cpp:36-193) on the level-0 grid.

There is no CPU fallback: if the CUDA library is missing or no GPU is
present, construction raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi as A

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libluma_gpu.so")

_lib = None


class LumaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"luma_gpu error {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the in-tree CUDA library (build it with ``luma_gb300.build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"luma_gb300 CUDA library not built: {LIB_PATH} missing "
                               "(run __graft_entry__.build() or python -m luma_gb300.build)")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.luma_gpu_abi_version.restype = C.c_int
        L.luma_gpu_last_error_string.restype = C.c_char_p
        L.luma_gpu_grid_create.argtypes = [C.POINTER(A.GridDesc), vp, C.POINTER(vp)]
        L.luma_gpu_grid_destroy.argtypes = [vp]
        L.luma_gpu_set_stream.argtypes = [vp, vp]
        L.luma_gpu_upload_state.argtypes = [vp, dp, dp, dp, dp, C.c_int]
        L.luma_gpu_download_state.argtypes = [vp, dp, dp, dp, dp]
        L.luma_gpu_get_time.argtypes = [vp, C.POINTER(C.c_int)]
        L.luma_gpu_step.argtypes = [vp, C.c_int]
        L.luma_gpu_synchronize.argtypes = [vp]
        L.luma_gpu_reduce.argtypes = [vp, C.POINTER(A.Reduction)]
        L.luma_gpu_planes_bytes.argtypes = [vp, C.c_int, C.POINTER(C.c_size_t)]
        L.luma_gpu_planes_export.argtypes = [vp, C.c_int, C.c_int, vp]
        L.luma_gpu_planes_import.argtypes = [vp, C.c_int, C.c_int, vp]
        L.luma_gpu_ibm_add_body.argtypes = [vp, C.c_int, dp, dp, C.POINTER(C.c_int)]
        L.luma_gpu_ibm_initialise.argtypes = [vp]
        L.luma_gpu_ibm_get_markers.argtypes = [vp, C.c_int, dp]
        L.luma_gpu_ibm_body_force.argtypes = [vp, C.c_int, dp]
        L.luma_gpu_ibm_add_filament.argtypes = [vp, dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                                C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                                C.POINTER(C.c_int)]
        L.luma_gpu_adj_forward.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp]
        L.luma_gpu_adj_backward.argtypes = [vp, C.c_double, dp, dp]
        L.luma_gpu_adj_memory.argtypes = [vp, C.POINTER(C.c_size_t)]
        L.luma_gpu_momex_force.argtypes = [vp, dp]
        L.luma_gpu_download_time_averages.argtypes = [vp, dp, dp, dp]
        L.luma_gpu_bfl_set.argtypes = [vp, C.POINTER(C.c_int32), C.c_int, dp]
        L.luma_gpu_bfl_forces.argtypes = [vp, dp]
        L.luma_gpu_io_lite.argtypes = [vp, C.c_char_p, C.c_double, C.c_int, C.c_int]
        L.luma_gpu_io_restart.argtypes = [vp, C.c_char_p, C.c_int]
        L.luma_gpu_io_wait.argtypes = [vp]
        L.luma_io_lite_write.argtypes = [C.POINTER(A.GridDesc), dp, dp, dp, dp, dp, dp, dp, C.c_char_p, C.c_double,
                                         C.c_int, C.c_int]
        L.luma_io_restart_write.argtypes = [C.POINTER(A.GridDesc), dp, dp, dp, C.c_char_p, C.c_int]
        L.luma_io_ibbody_restart_write.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), dp,
                                                   dp]
        L.luma_io_restart_read.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.POINTER(A.GridDesc)),
                                           C.POINTER(dp), C.POINTER(dp), C.POINTER(dp)]
        if L.luma_gpu_abi_version() != A.ABI_VERSION:
            raise RuntimeError("luma_gb300 library ABI version mismatch")
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != A.LUMA_OK:
        raise LumaError(rc, lib().luma_gpu_last_error_string().decode(errors="replace"))


class GpuGrid:
    """One grid of the device hierarchy.  Sub-grids are created with
    ``parent=``; only the level-0 grid is stepped, and destroying it frees
    the whole tree."""

    def __init__(self, desc: "A.GridDesc", parent: "GpuGrid | None" = None):
        self.L = lib()
        self.desc = desc
        h = C.c_void_p()
        check(self.L.luma_gpu_grid_create(C.byref(desc), parent.h if parent else None, C.byref(h)))
        self.h = h.value
        self.n = desc.N * desc.M * desc.K
        self.parent = parent
        self.children: list[GpuGrid] = []
        if parent is not None:
            parent.children.append(self)

    def close(self):
        if self.h and self.parent is None:
            self.L.luma_gpu_grid_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def planes_bytes(self, nplanes: int) -> int:
        v = C.c_size_t()
        check(self.L.luma_gpu_planes_bytes(self.h, nplanes, C.byref(v)))
        return v.value

    def planes_export(self, i0: int, nplanes: int, buf_ptr: int) -> None:
        """Current populations of x-planes i0.. (device storage, direction-major)
        into `buf_ptr` (device or pinned host address), on the grid's stream."""
        check(self.L.luma_gpu_planes_export(self.h, i0, nplanes, buf_ptr))

    def planes_import(self, i0: int, nplanes: int, buf_ptr: int) -> None:
        check(self.L.luma_gpu_planes_import(self.h, i0, nplanes, buf_ptr))

    def set_stream(self, stream_ptr: int | None):
        check(self.L.luma_gpu_set_stream(self.h, stream_ptr))

    def upload(self, f=None, u=None, rho=None, force=None, t: int = 0):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (f, u, rho, force)]
        check(self.L.luma_gpu_upload_state(self.h, *[A.dptr(a) for a in arrs], t))

    def download(self, f=True, u=True, rho=True, force=False) -> dict:
        d = self.desc
        out = {}
        bufs = []
        for name, want, size in (("f", f, self.n * d.Q), ("u", u, self.n * d.dims), ("rho", rho, self.n),
                                 ("force", force, self.n * d.dims)):
            arr = np.empty(size) if want else None
            if want:
                out[name] = arr
            bufs.append(A.dptr(arr))
        check(self.L.luma_gpu_download_state(self.h, *bufs))
        return out

    def step(self, nsteps: int = 1):
        check(self.L.luma_gpu_step(self.h, nsteps))

    def synchronize(self):
        check(self.L.luma_gpu_synchronize(self.h))

    @property
    def t(self) -> int:
        v = C.c_int()
        check(self.L.luma_gpu_get_time(self.h, C.byref(v)))
        return v.value

    def reduce(self) -> dict:
        r = A.Reduction()
        check(self.L.luma_gpu_reduce(self.h, C.byref(r)))
        return {"mass": r.mass, "momentum": tuple(r.momentum), "kinetic_energy": r.kinetic_energy,
                "max_speed": r.max_speed, "nonfinite": r.nonfinite}

    # ---- immersed-boundary bodies ----
    def ibm_add_body(self, positions, velocities=None) -> int:
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64).reshape(-1, 3)
        idx = C.c_int()
        check(self.L.luma_gpu_ibm_add_body(self.h, pos.shape[0], A.dptr(pos), A.dptr(vel), C.byref(idx)))
        self._nm = getattr(self, "_nm", []) + [pos.shape[0]]
        return idx.value

    def ibm_initialise(self):
        check(self.L.luma_gpu_ibm_initialise(self.h))

    def ibm_markers(self, body: int) -> np.ndarray:
        out = np.empty((self._nm[body], 9))
        check(self.L.luma_gpu_ibm_get_markers(self.h, body, A.dptr(out)))
        return out

    def ibm_body_force(self, body: int) -> np.ndarray:
        out = np.zeros(3)
        check(self.L.luma_gpu_ibm_body_force(self.h, body, A.dptr(out)))
        return out

    def ibm_add_filament(self, start, length, height, depth, angle_v, nel, clamped, density, E, dm,
                         fsi_vel_scale) -> int:
        import math
        st = np.ascontiguousarray(start, dtype=np.float64)
        idx = C.c_int()
        check(self.L.luma_gpu_ibm_add_filament(self.h, A.dptr(st), length, height, depth, angle_v, nel,
                                               int(clamped), density, E, dm, fsi_vel_scale, C.byref(idx)))
        self._nm = getattr(self, "_nm", []) + [int(math.floor(length / self.desc.dh)) + 1]
        return idx.value

    def time_averages(self) -> dict:
        """Running means (reference layout): rho (n), u (n*D), uu (n*(3D-3))."""
        d = self.desc
        n = d.N * d.M * d.K
        out = {"rho": np.zeros(n), "u": np.zeros(n * d.dims), "uu": np.zeros(n * (3 * d.dims - 3))}
        check(self.L.luma_gpu_download_time_averages(self.h, A.dptr(out["rho"]), A.dptr(out["u"]), A.dptr(out["uu"])))
        return out

    def momex_force(self) -> np.ndarray:
        """Momentum-exchange force of the solid sites (lattice units)."""
        out = np.zeros(3)
        check(self.L.luma_gpu_momex_force(self.h, A.dptr(out)))
        return out

    def bfl_set(self, site_marker, q) -> None:
        """BFL body 0: per-site marker of the site's voxel (-1 for none) and
        the (nmarkers, Q) link distances (-1: no wall on the link)."""
        sm = np.ascontiguousarray(site_marker, dtype=np.int32)
        q = np.ascontiguousarray(q, dtype=np.float64)
        self._bfl_nm = int(q.shape[0])
        check(self.L.luma_gpu_bfl_set(self.h, sm.ctypes.data_as(C.POINTER(C.c_int32)), self._bfl_nm, A.dptr(q)))

    def bfl_forces(self) -> np.ndarray:
        """(nmarkers, 3) momentum-exchange force per BFL marker of the latest step."""
        out = np.zeros((self._bfl_nm, 3))
        check(self.L.luma_gpu_bfl_forces(self.h, A.dptr(out)))
        return out

    # ---- output in the reference's formats ----
    def io_lite(self, directory: str, tval: float, precision: int = 10, rank: int = 0) -> None:
        """GridObj::io_lite for the tree (files written by a host thread)."""
        check(self.L.luma_gpu_io_lite(self.h, directory.encode(), float(tval), precision, rank))

    def io_restart(self, directory: str, rank: int = 0) -> None:
        """GridObj::io_restart(eWrite) for the tree (written by a host thread)."""
        check(self.L.luma_gpu_io_restart(self.h, directory.encode(), rank))

    def io_wait(self) -> None:
        check(self.L.luma_gpu_io_wait(self.h))

    # ---- discrete adjoint of the time-averaged drag ----
    def adj_forward(self, nsteps: int, checkpoint_every: int, body: int = 0) -> float:
        """Runs nsteps steps, checkpointing every checkpoint_every, and returns
        the time-averaged drag J of `body` (lattice units)."""
        J = C.c_double()
        check(self.L.luma_gpu_adj_forward(self.h, nsteps, checkpoint_every, body, C.byref(J)))
        self._adj_body = body
        return J.value

    def adj_backward(self, dJ: float = 1.0):
        """Returns (dJ/ds of the inlet velocity scale, dJ/dX as (markers, dims))."""
        gs = C.c_double()
        body = getattr(self, "_adj_body", 0)
        gx = np.zeros((self._nm[body], self.desc.dims))
        check(self.L.luma_gpu_adj_backward(self.h, dJ, C.byref(gs), A.dptr(gx)))
        return gs.value, gx

    def adj_memory(self) -> int:
        b = C.c_size_t()
        check(self.L.luma_gpu_adj_memory(self.h, C.byref(b)))
        return b.value


def write_io_lite(desc, f, fnew, u, rho, directory: str, tval: float, precision: int = 10, rank: int = 0,
                  averages: dict | None = None) -> None:
    """The io_lite format from host arrays (reference layout) of one grid;
    `averages` (keys rho, u, uu) adds the time-averaged columns."""
    tav = (averages["rho"], averages["u"], averages["uu"]) if averages else (None, None, None)
    arr = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None for x in (f, fnew, u, rho, *tav)]
    check(lib().luma_io_lite_write(C.byref(desc), *(A.dptr(x) for x in arr), directory.encode(), float(tval),
                                   precision, rank))


def write_io_restart(desc, f, u, rho, path: str, append: bool = False) -> None:
    """The io_restart format from host arrays (reference layout) of one grid."""
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (f, u, rho)]
    check(lib().luma_io_restart_write(C.byref(desc), *(A.dptr(x) for x in arr), path.encode(), int(append)))


def read_io_restart(path: str, descs, states) -> None:
    """GridObj::io_restart(eRead) into host arrays: descs (level 0 first) and
    states [{"f", "u", "rho"}] (float64, reference layout), overwritten in
    place."""
    n = len(descs)
    darr = (C.POINTER(A.GridDesc) * n)(*[C.pointer(d) for d in descs])
    for st in states:
        for k in ("f", "u", "rho"):
            assert st[k].dtype == np.float64 and st[k].flags["C_CONTIGUOUS"]
    fp = (C.POINTER(C.c_double) * n)(*[A.dptr(st["f"]) for st in states])
    up = (C.POINTER(C.c_double) * n)(*[A.dptr(st["u"]) for st in states])
    rp = (C.POINTER(C.c_double) * n)(*[A.dptr(st["rho"]) for st in states])
    check(lib().luma_io_restart_read(path.encode(), n, darr, fp, up, rp))


def write_io_ibbody_restart(path: str, positions, positions0=None) -> None:
    """The IB-body restart file: positions (one (n_b, 3) array per body);
    positions0 (same shapes, or None per body) marks flexible bodies."""
    nb = len(positions)
    counts = np.array([len(p) for p in positions], dtype=np.int32)
    flex = np.array([0 if positions0 is None or positions0[b] is None else 1 for b in range(nb)], dtype=np.int32)
    pos = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.float64).reshape(-1, 3) for p in positions])
                               if nb else np.zeros((0, 3)))
    pos0 = None
    if flex.any():
        pos0 = np.ascontiguousarray(np.concatenate([
            np.asarray(positions0[b] if flex[b] else positions[b], dtype=np.float64).reshape(-1, 3)
            for b in range(nb)]))
    ip = C.POINTER(C.c_int)
    check(lib().luma_io_ibbody_restart_write(path.encode(), nb, counts.ctypes.data_as(ip), flex.ctypes.data_as(ip),
                                             A.dptr(pos), A.dptr(pos0)))
