"""Slab decomposition along x on the GPU: the halo planes move through the
C ABI's plane export and import (luma_gpu_planes_export / _import), here
between slabs held by one process on one GPU.  After the steps, each
slab's real planes must equal, bit for bit, the same planes of the
undivided grid stepped with the same kernels (both grids take the
two-buffer step with the interior kernel at any size), in FP64 and in
shifted FP32; and FP64 must match the oracle within 1e-12.  The exchange
between ranks is checked on the host with gloo in test_slabs_cpu.py; runs
here have one GPU, so the NCCL transport is not run.
"""
import numpy as np
import pytest

from luma_gb300 import _abi as A
from luma_gb300 import slabs as S
from oracle import oracle as O
from tests.test_slabs_cpu import state, tgv_box, wall_channel

pytestmark = pytest.mark.gpu

FLAGS = A.FLAG_TWO_BUFFER | A.FLAG_SPLIT_INTERIOR


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED], ids=["fp64", "fp32s"])
@pytest.mark.parametrize("make,nslabs,steps", [(tgv_box, 2, 8), (tgv_box, 3, 5), (wall_channel, 4, 20)],
                         ids=["tgv_2", "tgv_3", "channel_4"])
def test_gpu_slabs_match_undivided_grid(make, nslabs, steps, prec):
    from luma_gb300.gpu import GpuGrid
    l0 = make()
    desc = l0.desc(precision=prec)
    desc.flags |= FLAGS
    whole = GpuGrid(desc)
    whole.upload(*state(l0), None, 0)
    whole.step(steps)
    want = whole.download()
    ranges = S.partition(l0.N, nslabs)
    slabs = []
    for a, b in ranges:
        lv = S.slab_level(l0, a, b)
        s = S.GpuSlab(lv, prec, flags=A.FLAG_SPLIT_INTERIOR)
        s.upload(*state(lv), None, 0)
        slabs.append(s)
    S.run(slabs, S.LocalExchange(slabs), steps)
    got = [s.download() for s in slabs]
    D, Q = l0.defs.dims, l0.defs.Q
    for key, per in (("f", Q), ("u", D), ("rho", 1)):
        assert np.array_equal(S.gather(l0, ranges, got, key, per), want[key]), key
    if prec == A.PREC_FP64:
        o = O.OracleGrid(l0.desc())
        o.upload(*state(l0), None, 0)
        o.step(steps)
        ref = o.download()
        u = S.gather(l0, ranges, got, "u", D)
        assert np.linalg.norm(u - ref["u"]) <= 1e-12 * np.linalg.norm(ref["u"])
    for s in slabs:
        s.close()
    whole.close()


def test_plane_transfer_refuses_in_place_grids_and_bad_planes():
    import torch
    from luma_gb300.gpu import GpuGrid, LumaError
    l0 = tgv_box(16)
    g = GpuGrid(l0.desc())                  # all-fluid periodic: the in-place step
    g.upload(*state(l0), None, 0)
    buf = torch.empty(g.planes_bytes(1), dtype=torch.uint8, device="cuda")
    with pytest.raises(LumaError, match="two-buffer"):
        g.planes_export(0, 1, buf.data_ptr())
    desc = l0.desc()
    desc.flags |= A.FLAG_TWO_BUFFER
    h = GpuGrid(desc)
    h.upload(*state(l0), None, 0)
    with pytest.raises(LumaError, match="off the grid"):
        h.planes_export(l0.N, 1, buf.data_ptr())
    g.close()
    h.close()
