"""CUDA path against the oracle and the reference's golden outputs.

FP64: relative L2 of u and rho <= 1e-10 against the oracle (which is
bit-exact with the reference), at every stored step of each oracle case.
FP32 shifted: relative L2 of u <= 2e-4 and |rho_32 - rho_64| <= 1e-5 on the
same cases, at the last stored step (the first for the KBC cases, whose
reference operator diverges).  The KBC cases are compared over the early steps the reference
stays finite on.
"""
import numpy as np
import pytest

from luma_gb300 import _abi as A
from oracle import oracle as O
from tests.golden import cases as CASES
from tests.golden import runner as R

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def gpu_grid(desc):
    from luma_gb300.gpu import GpuGrid
    return GpuGrid(desc)



def make_gpu(desc, parent):
    from luma_gb300.gpu import GpuGrid
    return GpuGrid(desc, parent)


def make_gpu_split(desc, parent):
    """Interior fluid sites in their own kernel at any grid size."""
    from luma_gb300.gpu import GpuGrid
    desc.flags |= A.FLAG_SPLIT_INTERIOR
    return GpuGrid(desc, parent)


def make_oracle(desc, parent):
    return O.OracleGrid(desc, parent)


NO_BODIES = sorted(n for n in CASES.CASES
                   if not CASES.CASES[n].get("bodies") and not CASES.CASES[n].get("filaments"))


@pytest.mark.parametrize("split", [False, True], ids=["one_kernel", "split_interior"])
@pytest.mark.parametrize("name", NO_BODIES)
def test_fp64_matches_oracle_and_reference(name, split):
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    gg, levels = R.build_backend(name, make_gpu_split if split else make_gpu, A.PREC_FP64)
    oo, _ = R.build_backend(name, make_oracle)
    done = 0
    for s in spec["steps"]:
        gg[0].step(s - done)
        oo[0].step(s - done)
        done = s
        gg[0].synchronize()
        for g, o, lv in zip(gg, oo, levels):
            key = R.grid_key(lv)
            gs, os_ = g.download(), o.download()
            assert g.t == o.t
            eu = rel_l2(gs["u"], os_["u"])
            er = rel_l2(gs["rho"], os_["rho"])
            ef = rel_l2(gs["f"], os_["f"])
            assert eu <= 1e-10 and er <= 1e-10 and ef <= 1e-10, (name, key, s, eu, er, ef)
            u, rho, *_ = R.fields_at(fx, key, s, name)
            if u is not None:  # and the reference's own fields
                assert rel_l2(gs["u"], u) <= 1e-10
                assert rel_l2(gs["rho"], rho) <= 1e-10


@pytest.mark.parametrize("split", [False, True], ids=["one_kernel", "split_interior"])
@pytest.mark.parametrize("name", NO_BODIES)
def test_fp32_shifted_close_to_fp64(name, split):
    spec = CASES.CASES[name]
    gg, levels = R.build_backend(name, make_gpu_split if split else make_gpu, A.PREC_FP32_SHIFTED)
    oo, _ = R.build_backend(name, make_oracle)
    s = spec["steps"][0] if name.startswith("kbc") else spec["steps"][-1]
    gg[0].step(s)
    oo[0].step(s)
    for g, o, lv in zip(gg, oo, levels):
        gs, os_ = g.download(), o.download()
        eu = rel_l2(gs["u"], os_["u"])
        dr = np.max(np.abs(gs["rho"] - os_["rho"]))
        assert eu <= 2e-4, (name, R.grid_key(lv), s, eu)
        assert dr <= 1e-5, (name, R.grid_key(lv), s, dr)


def test_aa_odd_and_even_step_counts():
    """The in-place path stores populations in two alternating layouts; f, u,
    rho must come back identical to the oracle after odd and even counts."""
    l0 = R.level0("tgv_d3q19")
    g = gpu_grid(l0.desc())
    o = O.OracleGrid(l0.desc())
    init = R.initial_state(l0)
    g.upload(*init, t=0)
    o.upload(*init, t=0)
    for n in (1, 2, 3, 5):
        g.step(n)
        o.step(n)
        gs, os_ = g.download(), o.download()
        assert rel_l2(gs["f"], os_["f"]) <= 1e-12
        assert rel_l2(gs["u"], os_["u"]) <= 1e-12
        assert rel_l2(gs["rho"], os_["rho"]) <= 1e-13


def test_reduce_mass_momentum():
    l0 = R.level0("tgv_d3q19")
    g = gpu_grid(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    g.step(4)
    st = g.download()
    red = g.reduce()
    assert red["nonfinite"] == 0
    assert abs(red["mass"] - st["rho"].sum()) <= 1e-9 * l0.ncell
    u = st["u"].reshape(-1, 3)
    mom = (st["rho"][:, None] * u).sum(axis=0)
    assert np.allclose(red["momentum"], mom, rtol=0, atol=1e-12 * l0.ncell)


@pytest.mark.parametrize("split", [False, True], ids=["one_kernel", "split_interior"])
@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("bodies")))
@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
def test_ibm_matches_oracle(name, prec, split):
    """Rigid IB bodies: supports/epsilon/ds from the host set-up equal the
    oracle's (bit-exact); marker forces and fields after the stored steps
    match at 1e-10 (FP64) or within the FP32 bounds."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    gg, levels = R.build_backend(name, make_gpu_split if split else make_gpu, prec)
    oo, _ = R.build_backend(name, make_oracle)
    oibm = O.OracleIBM()
    blev = CASES.bodies(name)[0][0]     # the grid that owns the body (level 1 on the refined sphere)
    for lev, reg, pos in CASES.bodies(name):
        gg[lev].ibm_add_body(pos)
        oibm.add_body(oo[lev], pos)
    gg[0].ibm_initialise()
    oibm.initialise()
    gm, om = gg[blev].ibm_markers(0), oibm.markers(0)
    assert np.array_equal(gm[:, 6:9], om[:, 6:9])
    assert np.array_equal(gm[:, 6], fx["markers_0"][:, 8])
    done = 0
    D = levels[0].defs.dims
    for s in spec["steps"]:
        gg[0].step(s - done)
        oo[0].step(s - done)
        done = s
        gm, om = gg[blev].ibm_markers(0), oibm.markers(0)
        ef = rel_l2(gm[:, 3:3 + D], om[:, 3:3 + D])
        for g, o, lv in zip(gg, oo, levels):
            gs, os_ = g.download(), o.download()
            eu = rel_l2(gs["u"], os_["u"])
            key = R.grid_key(lv)
            if prec == A.PREC_FP64:
                assert eu <= 1e-10 and rel_l2(gs["f"], os_["f"]) <= 1e-10, (name, key, s, eu)
                u_ref = R.fields_at(fx, key, s, name)[0]
                assert rel_l2(gs["u"], u_ref) <= 1e-10, (name, key, s)
            else:
                assert eu <= 2e-4, (name, key, s, eu)
        if prec == A.PREC_FP64:
            assert ef <= 1e-9, (name, s, ef)
            assert rel_l2(gm[:, 3:3 + D], fx[f"markers_{s}"][:, 5:5 + D]) <= 1e-9, (name, s)
        else:
            assert ef <= 1e-3, (name, s, ef)
    tot = gg[blev].ibm_body_force(0)
    mk = gg[blev].ibm_markers(0)
    vd = mk[:, 7] if D == 3 else 1.0
    ref = (mk[:, 3:3 + D] * (mk[:, 6] * vd * mk[:, 7])[:, None]).sum(axis=0)
    assert np.allclose(tot[:D], ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("filaments")))
def test_filament_fsi_matches_oracle(name):
    """Flexible filament with the FEM and the FSI sub-iterations on the
    device, FP64, against the oracle (bit-exact with the reference): flow
    field rel L2 <= 1e-10, marker positions within 1e-12, marker forces rel
    L2 <= 1e-8 after the stored steps."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    gg, levels = R.build_backend(name, make_gpu, A.PREC_FP64)
    oo, _ = R.build_backend(name, make_oracle)
    oibm = O.OracleIBM()
    R.attach_filaments(name, gg, levels, lambda g, **k: g.ibm_add_filament(**k))
    R.attach_filaments(name, oo, levels, lambda g, **k: oibm.add_filament(g, **k))
    gg[0].ibm_initialise()
    oibm.initialise()
    done = 0
    for s in spec["steps"]:
        gg[0].step(s - done)
        oo[0].step(s - done)
        done = s
        gs, os_ = gg[0].download(), oo[0].download()
        gm, om = gg[0].ibm_markers(0), oibm.markers(0)
        assert rel_l2(gs["u"], os_["u"]) <= 1e-10, (s, rel_l2(gs["u"], os_["u"]))
        assert np.max(np.abs(gm[:, 0:2] - om[:, 0:2])) <= 1e-12
        assert rel_l2(gm[:, 3:5], om[:, 3:5]) <= 1e-8, (s, rel_l2(gm[:, 3:5], om[:, 3:5]))
        assert rel_l2(gs["u"], fx[f"u_{s}"]) <= 1e-10


@pytest.mark.parametrize("split", [False, True], ids=["one_kernel", "split_interior"])
def test_filament_3d_matches_oracle(split):
    """A filament on a 3D grid (D3Q19 channel 40x20x10): the planar beam
    with the one change that lets it run in 3D (x-y load and marker update,
    markers keep z).  The reference aborts there, so parity is against the
    oracle only (3D FEM parity unpinned by the reference): FP64 flow field
    rel L2 <= 1e-10, marker positions within 1e-11, marker forces rel L2
    <= 1e-8 after 40 steps."""
    from luma_gb300 import case as hc
    V, X, S, F = A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.FLUID
    d = hc.Definitions(dims=3, resolution=20, timestep=1.0 / 500.0, bx=2.0, by=1.0, bz=0.5, re=100, ux0=1.0,
                       ibm=True, walls=(V, X, S, S, F, F))
    l0 = hc.build_level0(d)
    dh = 1.0 / d.resolution
    fil = dict(start=(0.513, dh, 0.261), length=0.4, height=0.02, depth=0.05, angle_v=90.0, nel=10,
               clamped=True, density=1.0e4, E=1.0e8, dm=(d.physical_rho / d.rho_in) * dh ** 3,
               fsi_vel_scale=d.ux0 * d.timestep / dh)
    desc = l0.desc(precision=A.PREC_FP64)
    if split:
        desc.flags |= A.FLAG_SPLIT_INTERIOR
    from luma_gb300.gpu import GpuGrid
    g = GpuGrid(desc)
    o = O.OracleGrid(l0.desc())
    f0 = hc.equilibrium(3, 19, l0.rho, l0.u).reshape(-1)
    for x in (g, o):
        x.upload(f0, l0.u, l0.rho, l0.force_xyz, 0)
    oibm = O.OracleIBM()
    g.ibm_add_filament(**fil)
    oibm.add_filament(o, **fil)
    g.ibm_initialise()
    oibm.initialise()
    for _ in range(4):
        g.step(10)
        o.step(10)
        gs, os_ = g.download(), o.download()
        gm, om = g.ibm_markers(0), oibm.markers(0)
        assert rel_l2(gs["u"], os_["u"]) <= 1e-10, rel_l2(gs["u"], os_["u"])
        assert np.max(np.abs(gm[:, 0:3] - om[:, 0:3])) <= 1e-11
        assert np.all(gm[:, 2] == fil["start"][2])
        assert rel_l2(gm[:, 3:6], om[:, 3:6]) <= 1e-8, rel_l2(gm[:, 3:6], om[:, 3:6])
    assert np.max(np.abs(gm[:, 0] - fil["start"][0])) > 1e-3   # the filament bent


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
def test_momentum_exchange_force(prec):
    """Momentum exchange over the solid sites: the Poiseuille channel's walls
    against the reference build's own L_LD_OUT force (tests/golden/
    make_momex.py) after 0..300 steps, and a channel with a bounce-back block
    against the oracle.  FP64: rel 1e-12 of the force magnitude; shifted
    FP32: 1e-5."""
    import json
    import os
    tol = 1e-12 if prec == A.PREC_FP64 else 1e-5
    ref = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "momex_d2q9.json")))
    gg, _ = R.build_backend(ref["like"], make_gpu, prec)
    for s in (1, 2, 50, 300):
        gg[0].step(s - 1 - gg[0].t)
        got, want = gg[0].momex_force(), np.array(ref["forces"][str(s)])
        scale = max(np.max(np.abs(want)), 1e-3)
        assert np.max(np.abs(got - want)) <= tol * scale, (s, got, want)
    # a bounce-back block in the channel (solid sites labelled on the host)
    from luma_gb300 import case as hc
    l0 = R.level0("poiseuille_d2q9")
    typ = l0.typ.reshape(l0.N, l0.M, l0.K).copy()
    typ[60:70, 45:55, :] = A.SOLID
    l0.typ = typ.reshape(-1)
    u = l0.u.reshape(l0.N, l0.M, l0.K, -1).copy()
    u[60:70, 45:55] = 0.0
    l0.u = u.reshape(-1)
    f0 = hc.equilibrium(2, 9, l0.rho, l0.u).reshape(-1)
    g = gpu_grid(l0.desc(precision=prec))
    o = O.OracleGrid(l0.desc())
    for x in (g, o):
        x.upload(f0, l0.u, l0.rho, None, 0)
    g.step(400)
    o.step(400)
    got, want = g.momex_force(), o.momex_force()
    assert abs(want[0]) > 1e-3
    assert np.max(np.abs(got - want)) <= tol * np.max(np.abs(want)), (got, want)


@pytest.mark.parametrize("split", [False, True], ids=["one_kernel", "split_interior"])
@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("bfl")))
def test_bfl_marker_forces(name, prec, split):
    """BFL cylinder (2D) and sphere (3D): per-marker momentum-exchange forces
    against the reference build's computeLiftDrag(v, id, g, markerID) at
    every stored step (FP64: within 1e-10 of the largest force, at least
    1e-3; shifted FP32: 1e-4)."""
    fx = R.fixture(name)
    tol = 1e-10 if prec == A.PREC_FP64 else 1e-4
    gg, _ = R.build_backend(name, make_gpu_split if split else make_gpu, prec)
    for s, want in zip(fx["bfl_force_steps"], fx["bfl_forces"]):
        gg[0].step(int(s) - gg[0].t)
        got = gg[0].bfl_forces()
        # a marker at rest in 3D carries a force that cancels to rounding:
        # the bound is relative to at least 1e-3 (a link carries ~2 w rho)
        scale = max(np.max(np.abs(want)), 1e-3)
        assert np.max(np.abs(got - want)) <= tol * scale, (int(s), np.max(np.abs(got - want)), scale)


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("store_tav")))
def test_time_averages_match_oracle(name, prec):
    """Running means on every grid at every stored step against the oracle
    (bit-exact with the reference): FP64 rel L2 <= 1e-10, shifted FP32 <= 2e-4
    for u and u u, 1e-6 for rho."""
    spec = CASES.CASES[name]
    gg, levels = R.build_backend(name, make_gpu, prec)
    oo, _ = R.build_backend(name, make_oracle)
    if spec.get("bodies"):
        ibm = O.OracleIBM()
        for (lev, reg, pos) in CASES.bodies(name):
            gg[lev].ibm_add_body(pos)
            ibm.add_body(oo[lev], pos)
        gg[0].ibm_initialise()
        ibm.initialise()
    tol = (1e-10, 1e-10) if prec == A.PREC_FP64 else (1e-6, 2e-4)
    done = 0
    for s in spec["steps"]:
        gg[0].step(s - done)
        oo[0].step(s - done)
        done = s
        for g, o, lv in zip(gg, oo, levels):
            a, b = g.time_averages(), o.time_averages()
            assert rel_l2(a["rho"], b["rho"]) <= tol[0], (R.grid_key(lv), s)
            assert rel_l2(a["u"], b["u"]) <= tol[1], (R.grid_key(lv), s)
            assert rel_l2(a["uu"], b["uu"]) <= tol[1], (R.grid_key(lv), s)


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
def test_pinned_host_arrays_transfer_in_place(prec):
    """Pinned host arrays are read and written in place by the layout
    conversions (no staging copy): the state they carry up and back equals
    the staged transfer of the same values in ordinary host memory."""
    import ctypes as C
    import torch
    from luma_gb300.gpu import check, lib
    L = lib()
    lv = R.level0("refine_d2q9")
    f0, u0, r0, _ = R.initial_state(lv)
    ga, gb = gpu_grid(lv.desc(precision=prec)), gpu_grid(lv.desc(precision=prec))
    ga.upload(f0, u0, r0, None, 0)
    pin = {k: torch.from_numpy(v.copy()).pin_memory() for k, v in (("f", f0), ("u", u0), ("rho", r0))}
    dp = C.POINTER(C.c_double)
    ptr = lambda t: C.cast(t.data_ptr(), dp)  # noqa: E731
    check(L.luma_gpu_upload_state(C.c_void_p(gb.h), ptr(pin["f"]), ptr(pin["u"]), ptr(pin["rho"]), None, 0))
    for g in (ga, gb):
        g.step(7)
        g.synchronize()
    want = ga.download()
    out = {k: torch.empty(v.size, dtype=torch.float64).pin_memory() for k, v in want.items() if k != "force"}
    check(L.luma_gpu_download_state(C.c_void_p(gb.h), ptr(out["f"]), ptr(out["u"]), ptr(out["rho"]), None))
    for k in ("f", "u", "rho"):
        assert np.array_equal(out[k].numpy(), want[k]), k
    ga.close()
    gb.close()
