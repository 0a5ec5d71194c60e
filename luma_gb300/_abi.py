"""ctypes mirror of ``include/luma_gpu.h`` (the ABI version is ``ABI_VERSION`` below).

The structure layouts here must match the header field for field; a CPU
test checks the sizes against the compiled library's own view.
"""
from __future__ import annotations

import ctypes as C

ABI_VERSION = 2

LUMA_OK = 0
LUMA_E_INVALID = -1
LUMA_E_CUDA = -2
LUMA_E_NOMEM = -3
LUMA_E_STATE = -4
LUMA_E_TIMEOUT = -5
LUMA_E_NUMERIC = -6
LUMA_E_DOMAIN = -7

# Site labels: values of the reference's eType (inc/Enumerations.h:84-96).
SOLID, FLUID, REFINED, TL_TO_COARSER, TL_TO_FINER, BFL, VELOCITY, PRESSURE, SLIP, \
    EXTRAPOLATE_RIGHT = range(10)

PREC_FP64 = 0
PREC_FP32_SHIFTED = 1

COLL_BGK = 0
COLL_BGK_SMAG = 1
COLL_KBC = 2

FLAG_REGULARISED = 0x1
FLAG_IBM = 0x2
FLAG_GRAVITY = 0x4
FLAG_FIX_MACRO3D = 0x8
FLAG_FIX_KBC = 0x10
FLAG_TWO_BUFFER = 0x20
FLAG_SPLIT_INTERIOR = 0x40
FLAG_TIME_AVERAGES = 0x80
FLAG_UNIVERSAL_EPSILON = 0x100

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class GridDesc(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int),
        ("level", C.c_int), ("region", C.c_int),
        ("dims", C.c_int), ("Q", C.c_int),
        ("N", C.c_int), ("M", C.c_int), ("K", C.c_int),
        ("precision", C.c_int),
        ("collision", C.c_int),
        ("flags", C.c_int),
        ("omega", C.c_double), ("dt", C.c_double), ("dh", C.c_double),
        ("refinement_ratio", C.c_double),
        ("rho_in", C.c_double),
        ("velocity_ramp", C.c_double),
        ("pressure_delta", C.c_double),
        ("gravity", C.c_double),
        ("gravity_dir", C.c_int),
        ("csmag", C.c_double),
        ("global_edges", C.c_double * 6),
        ("wall_thickness", C.c_double * 6),
        ("coarse_lims", C.c_int * 6),
        ("lattyp", _ip),
        ("xpos", _dp), ("ypos", _dp), ("zpos", _dp),
        ("ux_in", _dp), ("uy_in", _dp), ("uz_in", _dp),
        ("reynolds_ramp", C.c_double), ("re", C.c_double),
    ]


class Reduction(C.Structure):
    _fields_ = [
        ("mass", C.c_double),
        ("momentum", C.c_double * 3),
        ("kinetic_energy", C.c_double),
        ("max_speed", C.c_double),
        ("nonfinite", C.c_int64),
    ]


def dptr(a):
    """Pointer to a contiguous float64 numpy array (or NULL for None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_ip)
