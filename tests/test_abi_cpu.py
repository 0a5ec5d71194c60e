"""CPU checks of the C ABI library: it loads, exports every entry point the
header declares, and its struct layout matches the ctypes mirror.  No
compute call is made (no GPU here)."""
import ctypes as C
import os
import re

import pytest

from luma_gb300 import _abi as A

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "luma_gpu.h")
LIB = os.path.join(ROOT, "luma_gb300", "_build", "libluma_gpu.so")


def declarations():
    """(name, [parameter declarations]) of every function the header
    declares."""
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = []
    for m in re.finditer(r"^\s*(?:int|const char \*)\s*(luma_\w+)\s*\(([^)]*)\)\s*;", src, re.M):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out.append((m.group(1), params))
    return out


def declared_functions():
    return sorted({name for name, _ in declarations()})


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from luma_gb300 import build
        build.build()
    try:
        return C.CDLL(LIB)
    except OSError as e:  # libcudart missing on a host without the toolkit
        pytest.skip(f"cannot load CUDA library here: {e}")


def test_header_declares_entry_points():
    names = declared_functions()
    assert "luma_gpu_step" in names and "luma_gpu_grid_create" in names
    assert len(names) >= 11


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def _ctype(param: str):
    if "*" in param or "[" in param:
        return C.c_void_p
    if param.startswith("double"):
        return C.c_double
    if param.startswith("size_t"):
        return C.c_size_t
    if param.startswith("int64_t"):
        return C.c_int64
    assert param.startswith("int"), param
    return C.c_int


# entry points for which every argument zero or null is a valid call
NULL_OK = {"luma_gpu_grid_destroy", "luma_gpu_abi_version", "luma_gpu_last_error_string"}


def test_every_entry_point_refuses_null_arguments(lib):
    """With every pointer null and every number zero, each entry point
    returns an error status (no CUDA call happens first, so this runs on a
    host without a GPU) and sets a message; destroying a null grid is a
    no-op."""
    lib.luma_gpu_last_error_string.restype = C.c_char_p
    names = []
    for name, params in declarations():
        if name in NULL_OK:
            continue
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [_ctype(p) for p in params]
        args = [None if t is C.c_void_p else 0 for t in fn.argtypes]
        rc = fn(*args)
        assert rc in (A.LUMA_E_INVALID, A.LUMA_E_STATE), (name, rc)
        assert lib.luma_gpu_last_error_string(), name
        names.append(name)
    assert len(names) >= 28
    lib.luma_gpu_grid_destroy.argtypes = [C.c_void_p]
    assert lib.luma_gpu_grid_destroy(None) == A.LUMA_OK


def test_abi_version_and_error_string(lib):
    lib.luma_gpu_abi_version.restype = C.c_int
    assert lib.luma_gpu_abi_version() == A.ABI_VERSION
    lib.luma_gpu_last_error_string.restype = C.c_char_p
    assert isinstance(lib.luma_gpu_last_error_string(), bytes)


def test_invalid_descriptor_rejected_without_gpu(lib):
    """Descriptor validation runs before any CUDA call: a wrong ABI version,
    an unsupported lattice, 3D KBC off D3Q27, more sites than 32-bit ids
    address and empty or 2D-with-depth grids come back as LUMA_E_INVALID."""
    lib.luma_gpu_grid_create.argtypes = [C.POINTER(A.GridDesc), C.c_void_p, C.POINTER(C.c_void_p)]
    lib.luma_gpu_last_error_string.restype = C.c_char_p
    d = A.GridDesc()
    d.abi_version = 999
    h = C.c_void_p()
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert b"ABI" in lib.luma_gpu_last_error_string()
    d.abi_version = A.ABI_VERSION
    d.dims, d.Q, d.N, d.M, d.K = 3, 15, 4, 4, 4
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert b"lattice" in lib.luma_gpu_last_error_string()
    d.Q = 19
    d.collision = A.COLL_KBC
    d.omega = 1.5
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert b"D3Q27" in lib.luma_gpu_last_error_string()
    # site ids are 32-bit: at most 2^31-1 sites per grid (1291^3 is above)
    d.N = d.M = d.K = 1291
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert b"2^31-1" in lib.luma_gpu_last_error_string()
    d.N, d.M, d.K = 0, 4, 4
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert b"bad grid size" in lib.luma_gpu_last_error_string()
    d.dims, d.Q, d.N, d.M, d.K = 2, 9, 4, 4, 2  # 2D grids have K = 1
    assert lib.luma_gpu_grid_create(C.byref(d), None, C.byref(h)) == A.LUMA_E_INVALID
    assert not h.value


def test_desc_struct_size_matches_header():
    """sizeof(luma_grid_desc) from a C compile of the header equals ctypes'."""
    import subprocess
    import tempfile
    src = '#include "luma_gpu.h"\n#include <stdio.h>\nint main(){printf("%zu %zu\\n", sizeof(luma_grid_desc), sizeof(luma_reduction));return 0;}\n'
    with tempfile.TemporaryDirectory() as td:
        c = os.path.join(td, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(td, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == C.sizeof(A.GridDesc)
    assert int(out[1]) == C.sizeof(A.Reduction)


def test_every_entry_point_cites_what_it_replaces():
    """The comment that documents each declared function (the nearest
    block comment above it, which a group of functions may share) names the
    reference interface the entry point replaces by file (src/... or
    inc/...), or states that it has no counterpart in the reference."""
    src = open(HEADER).read()
    cite = re.compile(r"\b(?:src|inc)/\w+\.(?:cpp|h)|no counterpart in the reference", re.I)
    missing = []
    for name in declared_functions():
        m = re.search(r"^\s*(?:int|const char \*)\s*" + name + r"\s*\(", src, re.M)
        assert m, name
        comments = list(re.finditer(r"/\*.*?\*/", src[:m.start()], re.S))
        # skip section rulers ("/* ---- name ---- */") to the comment that documents the call
        doc = next((c.group(0) for c in reversed(comments) if not re.match(r"/\* -{3,}", c.group(0))), "")
        if not cite.search(doc):
            missing.append(name)
    assert not missing, missing
