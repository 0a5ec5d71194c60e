"""The no-allocation reduction entry point, through the C ABI.

luma_gpu_reduce_fields_noalloc serves callers that cannot allocate device
memory (hosts that give the GPU's memory to a fixed pool at start-up,
real-time loops that cannot afford an allocation).  It must give the same
FP64 sums as luma_gpu_reduce on the same fields — here within the FP64
parity tolerance of these tests (relative 1e-10) — on two calls in a row,
because both calls share the entry point's fixed scratch array; the second
call must leave the device's free memory unchanged; and it must refuse a
size beyond its stated maximum with a clear error, and a stream under
capture.

This file is collected last so that a stop-at-first-failure run has already
run every other test; it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from luma_gb300 import _abi as A
from tests.golden import runner as R

pytestmark = pytest.mark.gpu

MAX_SITES = 16_777_216


def _lib():
    from luma_gb300.gpu import lib
    L = lib()
    L.luma_gpu_reduce_fields_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int,
                                                 C.c_void_p, C.POINTER(A.Reduction)]
    return L


def _close(got: A.Reduction, ref: dict, n: int):
    tol = 1e-10
    assert got.nonfinite == ref["nonfinite"] == 0
    assert abs(got.mass - ref["mass"]) <= tol * abs(ref["mass"])
    scale = max(abs(ref["mass"]), 1.0)
    for d in range(3):
        assert abs(got.momentum[d] - ref["momentum"][d]) <= tol * scale
    assert abs(got.kinetic_energy - ref["kinetic_energy"]) <= tol * max(abs(ref["kinetic_energy"]), 1e-300)
    assert abs(got.max_speed - ref["max_speed"]) <= tol * max(ref["max_speed"], 1e-300)


@pytest.mark.parametrize("name", ["tgv_d3q19", "poiseuille_d2q9"])
def test_noalloc_reduction_matches_reduce(name):
    import torch
    from luma_gb300.gpu import GpuGrid, check

    L = _lib()
    lv = R.level0(name)
    g = GpuGrid(lv.desc(precision=A.PREC_FP64))
    g.upload(*R.initial_state(lv), t=0)
    g.step(3)
    g.synchronize()
    ref = g.reduce()
    st = g.download(f=False)
    D = lv.defs.dims
    n = lv.ncell
    dev = torch.device("cuda", 0)
    typ = torch.from_numpy(lv.typ.astype(np.uint8)).to(dev)
    rho = torch.from_numpy(st["rho"]).to(dev)
    u = torch.from_numpy(np.ascontiguousarray(st["u"].reshape(n, D).T)).to(dev)  # SoA u[d][id]
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    for call in range(2):  # two calls in a row share the scratch array
        free0 = torch.cuda.mem_get_info(dev)[0]
        out = A.Reduction()
        check(L.luma_gpu_reduce_fields_noalloc(typ.data_ptr(), rho.data_ptr(), u.data_ptr(), n, D,
                                               stream.cuda_stream, C.byref(out)))
        _close(out, ref, n)
        if call == 1:   # the first call may load the module's code; the second allocates nothing
            assert torch.cuda.mem_get_info(dev)[0] == free0
    g.close()


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch
    L = _lib()
    dev = torch.device("cuda", 0)
    small = torch.zeros(16, dtype=torch.float64, device=dev)
    typ = torch.ones(16, dtype=torch.uint8, device=dev)
    out = A.Reduction()
    rc = L.luma_gpu_reduce_fields_noalloc(typ.data_ptr(), small.data_ptr(), small.data_ptr(), MAX_SITES + 1, 3,
                                          None, C.byref(out))
    assert rc == A.LUMA_E_INVALID
    msg = L.luma_gpu_last_error_string().decode()
    assert "at most 16777216 sites" in msg


def test_noalloc_refuses_a_stream_under_capture():
    """The call copies its sums to the host and waits on the stream, which a
    capturing stream cannot do: it is refused with LUMA_E_INVALID before
    anything is recorded, the capture completes and replays, and the same
    stream takes the call once the capture has ended."""
    import torch
    L = _lib()
    dev = torch.device("cuda", 0)
    n = 5000
    typ = torch.full((n,), 1, dtype=torch.uint8, device=dev)          # LUMA_SITE_FLUID
    rho = torch.full((n,), 1.25, dtype=torch.float64, device=dev)
    u = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    y = torch.zeros(n, dtype=torch.float64, device=dev)
    s = torch.cuda.Stream(dev)
    out = A.Reduction()
    with torch.cuda.stream(s):    # the device's scratch address is looked up outside the capture
        assert L.luma_gpu_reduce_fields_noalloc(typ.data_ptr(), rho.data_ptr(), u.data_ptr(), n, 3,
                                                s.cuda_stream, C.byref(out)) == A.LUMA_OK
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        rc = L.luma_gpu_reduce_fields_noalloc(typ.data_ptr(), rho.data_ptr(), u.data_ptr(), n, 3,
                                              s.cuda_stream, C.byref(out))
        y.copy_(rho * 2.0)
    assert rc == A.LUMA_E_INVALID
    assert "under capture" in L.luma_gpu_last_error_string().decode()
    graph.replay()
    torch.cuda.synchronize(dev)
    assert float(y.sum()) == 2.5 * n
    out = A.Reduction()
    from luma_gb300.gpu import check
    check(L.luma_gpu_reduce_fields_noalloc(typ.data_ptr(), rho.data_ptr(), u.data_ptr(), n, 3,
                                           s.cuda_stream, C.byref(out)))
    assert out.mass == 1.25 * n and out.nonfinite == 0 and out.max_speed == 0.0
