"""Slab decomposition along x (luma_gb300/slabs.py), on the host.

The decomposition replaces the reference's MPI sub-domains and their halo
exchange (MpiManager::mpi_communicate, src/MpiManager.cpp:631-820).  Here
the slabs are oracle grids, so the partition, the ghost planes, the
neighbour ring and the messages are checked without a GPU: after every step
each slab's real planes must equal, bit for bit, the same planes of the
undivided grid stepped alone.  Two transports: the slabs of one process
(``LocalExchange``) and one slab per process over two gloo ranks
(``DistExchange``).  The device side of the exchange (the plane export and
import of the C ABI) is checked on the GPU in test_gpu_slabs.py.
"""
import json
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from luma_gb300 import _abi as A  # noqa: E402
from luma_gb300 import case as hostcase  # noqa: E402
from luma_gb300 import slabs as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.golden import cases as CASES  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def tgv_box(n=24, nz=None):
    d = hostcase.Definitions(dims=3, resolution=n, timestep=1.0 / (16 * n), bx=1.0, by=1.0, bz=(nz or n) / n,
                             re=300, walls=(A.FLUID,) * 6)
    l0 = hostcase.build_level0(d)
    l0.u = CASES.taylor_green(l0.N, l0.M, l0.K, 0.02, 1e-4).reshape(-1)
    return l0


def wall_channel():
    """D2Q9, periodic in x, solid bottom/top walls, a shear start."""
    d = hostcase.Definitions(dims=2, resolution=20, timestep=1.0 / 400.0, bx=2.0, by=1.0, re=50,
                             walls=(A.FLUID, A.FLUID, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    l0 = hostcase.build_level0(d)
    u = l0.u.reshape(l0.N, l0.M, 1, 2)
    y = (np.arange(l0.M) + 0.5) / l0.M
    u[..., 0] = (0.03 * np.sin(np.pi * y))[None, :, None]
    u[..., 1] = (0.01 * np.sin(2 * np.pi * (np.arange(l0.N) + 0.5) / l0.N))[:, None, None]
    l0.u = u.reshape(-1)
    return l0


def state(lv):
    f0 = hostcase.equilibrium(lv.defs.dims, lv.defs.Q, lv.rho, lv.u).reshape(-1)
    return f0, lv.u.copy(), lv.rho.copy()


def undivided(l0, steps):
    g = O.OracleGrid(l0.desc())
    g.upload(*state(l0), None, 0)
    g.step(steps)
    return g.download()


def host_slabs(l0, nslabs):
    ranges = S.partition(l0.N, nslabs)
    out = []
    for a, b in ranges:
        lv = S.slab_level(l0, a, b)
        s = S.HostSlab(lv, O.OracleGrid(lv.desc()))
        s.upload(*state(lv), None, 0)
        out.append(s)
    return ranges, out


def test_partition_and_ghost_planes():
    assert S.partition(10, 3) == [(0, 4), (4, 7), (7, 10)]
    assert list(S.ghost_planes(10, 0, 4)) == [9, 0, 1, 2, 3, 4]
    assert list(S.ghost_planes(10, 7, 10)) == [6, 7, 8, 9, 0]
    with pytest.raises(ValueError):
        S.partition(3, 4)


def test_slabs_refuse_boundary_conditions_across_a_cut():
    d = hostcase.Definitions(dims=2, resolution=10, timestep=1.0 / 200.0, bx=2.0, by=1.0, re=50, ux0=1.0,
                             walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    with pytest.raises(ValueError):
        S.slab_level(hostcase.build_level0(d), 0, 10)


@pytest.mark.parametrize("make,nslabs,steps", [(tgv_box, 2, 6), (tgv_box, 3, 4), (wall_channel, 4, 12)],
                         ids=["tgv_2", "tgv_3", "channel_4"])
def test_local_slabs_match_undivided_grid(make, nslabs, steps):
    l0 = make()
    want = undivided(l0, steps)
    ranges, slabs = host_slabs(l0, nslabs)
    S.run(slabs, S.LocalExchange(slabs), steps)
    got = [s.download() for s in slabs]
    D, Q = l0.defs.dims, l0.defs.Q
    for key, per in (("f", Q), ("u", D), ("rho", 1)):
        assert np.array_equal(S.gather(l0, ranges, got, key, per), want[key]), key


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    l0 = tgv_box(20)
    a, b = S.partition(l0.N, world)[rank]
    lv = S.slab_level(l0, a, b)
    slab = S.HostSlab(lv, O.OracleGrid(lv.desc()))
    slab.upload(*state(lv), None, 0)
    S.run(slab, S.DistExchange(slab, rank, world), 5)
    st = slab.download()
    np.save(os.path.join(out_dir, f"f{rank}.npy"), st["f"])
    np.save(os.path.join(out_dir, f"u{rank}.npy"), st["u"])
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fp:
        json.dump({"range": [a, b], "t": slab.grid.t}, fp)
    dist.barrier()
    dist.destroy_process_group()


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_gloo_ranks_match_undivided_grid(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    l0 = tgv_box(20)
    want = undivided(l0, 5)
    meta = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    ranges = [tuple(m["range"]) for m in meta]
    assert all(m["t"] == 5 for m in meta)
    got = [{"f": np.load(tmp_path / f"f{r}.npy"), "u": np.load(tmp_path / f"u{r}.npy")} for r in range(world)]
    assert np.array_equal(S.gather(l0, ranges, got, "f", 19), want["f"])
    assert np.array_equal(S.gather(l0, ranges, got, "u", 3), want["u"])
