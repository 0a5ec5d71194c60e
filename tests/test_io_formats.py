"""Writers in the reference's ASCII formats (GridObj::io_lite, io_restart).

CPU: the library's writers fed with the oracle's state (bit-exact with the
reference) reproduce the files the reference's own writers produced on the
same case byte for byte (SHA-256, tests/golden/make_io.py).
GPU: the asynchronous snapshot writers on the device state (FP64) give the
same layout, and values within one unit of the last printed digit; the
IB-body restart file byte for byte (rigid bodies) or equal to the host
writer's on the device's marker positions (a filament).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden import runner as R

HERE = os.path.dirname(os.path.abspath(__file__))
CASES_IO = ("refine_d2q9", "tavg_refine_d2q9", "ibm_cyl_d2q9")  # time averages; an IB cylinder


def ref_of(case):
    return json.load(open(os.path.join(HERE, "golden", f"io_{case}.json")))


def oracle_files(tmp_path, REF):
    from luma_gb300 import gpu as G
    from tests.golden import cases as CASE_DEFS
    grids, levels = R.build_backend(REF["case"], lambda d, p: O.OracleGrid(d, p))
    bodies = CASE_DEFS.bodies(REF["case"])
    if bodies:
        ibm = O.OracleIBM()
        for lev, reg, pos in bodies:
            ibm.add_body(grids[lev], pos)
        ibm.initialise()
    grids[0].step(REF["steps"])
    if bodies:
        mk = [ibm.markers(b) for b in range(len(bodies))]
        G.write_io_ibbody_restart(os.path.join(tmp_path, "restart_IBBody_Rnk0.out"),
                                  [m[:, 0:3] for m in mk])
    restart = os.path.join(tmp_path, "restart_LBM_Rnk0.out")
    for n, (g, lv) in enumerate(zip(grids, levels)):
        st = g.download()
        desc = lv.desc()
        tav = g.time_averages() if lv.defs.time_averages else None
        G.write_io_lite(desc, st["f"], g.fnew(), st["u"], st["rho"], str(tmp_path), REF["steps"], REF["precision"],
                        averages=tav)
        G.write_io_restart(desc, st["f"], st["u"], st["rho"], restart, append=n > 0)
    return tmp_path


@pytest.mark.parametrize("case", CASES_IO)
def test_writers_reproduce_reference_files(tmp_path, case):
    REF = ref_of(case)
    out = oracle_files(tmp_path, REF)
    for name, ref in REF["files"].items():
        data = open(os.path.join(out, name), "rb").read()
        assert len(data) == ref["bytes"], name
        assert hashlib.sha256(data).hexdigest() == ref["sha256"], name


def _rows(path):
    with open(path) as fp:
        return [line.rstrip("\n").split("\t") for line in fp]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES_IO)
def test_gpu_snapshot_writers_match_oracle(tmp_path, case):
    """The same files from the device state; with IB bodies the restart also
    writes restart_IBBody (rigid markers keep their positions, so that file
    is the reference's byte for byte)."""
    from luma_gb300 import _abi as A
    from luma_gb300.gpu import GpuGrid
    from tests.golden import cases as CASE_DEFS
    REF = ref_of(case)
    ref_dir = tmp_path / "ref"
    gpu_dir = tmp_path / "gpu"
    ref_dir.mkdir()
    gpu_dir.mkdir()
    oracle_files(ref_dir, REF)
    gg, _ = R.build_backend(REF["case"], lambda d, p: GpuGrid(d, p), A.PREC_FP64)
    bodies = CASE_DEFS.bodies(REF["case"])
    for lev, reg, pos in bodies:
        gg[lev].ibm_add_body(pos)
    if bodies:
        gg[0].ibm_initialise()
    gg[0].step(REF["steps"])
    gg[0].io_lite(str(gpu_dir), REF["steps"], REF["precision"])
    gg[0].io_restart(str(gpu_dir))
    gg[0].step(3)          # the GPU steps on while the host thread writes
    gg[0].io_wait()
    for name in REF["files"]:
        if name.startswith("restart_IBBody"):
            data = open(gpu_dir / name, "rb").read()
            assert hashlib.sha256(data).hexdigest() == REF["files"][name]["sha256"], name
            continue
        a, b = _rows(gpu_dir / name), _rows(ref_dir / name)
        assert len(a) == len(b), name
        for ra, rb in zip(a, b):
            assert len(ra) == len(rb)
            assert ra[:2] == rb[:2]           # rank/level and label/region
            # one unit in the last printed digit: 10 decimals (io_lite), 6
            # significant digits (restart)
            tol = dict(rtol=0.0, atol=2e-10) if name.startswith("io_lite") else dict(rtol=2e-5, atol=1e-9)
            assert np.allclose(np.array(ra[2:-1], float), np.array(rb[2:-1], float), **tol), name


@pytest.mark.gpu
def test_gpu_restart_lists_filament_markers(tmp_path):
    """A filament's entry in restart_IBBody: the marker positions the FEM has
    moved on the device, then the markers' initial positions (the
    reference's IBMarker::position0); the file equals the host writer's on
    the positions the device reports."""
    from luma_gb300 import _abi as A
    from luma_gb300 import gpu as G
    from luma_gb300.gpu import GpuGrid
    from tests.golden import cases as CASE_DEFS
    name = sorted(n for n in CASE_DEFS.CASES if CASE_DEFS.CASES[n].get("filaments"))[0]
    gg, levels = R.build_backend(name, lambda d, p: GpuGrid(d, p), A.PREC_FP64)
    idx = R.attach_filaments(name, gg, levels, lambda g, **k: g.ibm_add_filament(**k))
    gg[0].ibm_initialise()
    start = [gg[0].ibm_markers(b)[:, 0:3].copy() for b in idx]
    gg[0].step(20)
    gg[0].io_restart(str(tmp_path))
    gg[0].io_wait()
    now = [gg[0].ibm_markers(b)[:, 0:3] for b in idx]
    assert any(not np.array_equal(a, b) for a, b in zip(now, start))   # the filament moved
    G.write_io_ibbody_restart(str(tmp_path / "host.out"), now, start)
    assert open(tmp_path / "restart_IBBody_Rnk0.out", "rb").read() == open(tmp_path / "host.out", "rb").read()


@pytest.mark.parametrize("case", CASES_IO)
def test_restart_reader_matches_reference(tmp_path, case):
    """The restart file read back (GridObj::io_restart(eRead): f rebuilt as
    feq (1 + dt f_neq / omega), with feq from level 0's state at the level-0
    index of every line, level 0's omega) gives every grid the f, u and rho
    the reference's own reader leaves (SHA-256 of the arrays)."""
    from luma_gb300 import gpu as G
    REF = ref_of(case)
    oracle_files(tmp_path, REF)
    levels = R.hierarchy(REF["case"])
    descs = [lv.desc() for lv in levels]
    states = []
    for lv in levels:
        f0, u0, rho0, _ = R.initial_state(lv)
        states.append({"f": f0.astype(np.float64).copy(), "u": np.ascontiguousarray(u0, dtype=np.float64),
                       "rho": np.ascontiguousarray(rho0, dtype=np.float64)})
    G.read_io_restart(os.path.join(tmp_path, "restart_LBM_Rnk0.out"), descs, states)
    for lv, st in zip(levels, states):
        key = R.grid_key(lv)
        for k in ("f", "u", "rho"):
            got = hashlib.sha256(np.ascontiguousarray(st[k]).tobytes()).hexdigest()
            assert got == REF["restart_read"][f"{key}_{k}"], (key, k)
