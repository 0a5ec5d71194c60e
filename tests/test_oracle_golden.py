"""The CPU oracle against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py from the reference's serial build)."""
import json
import os

import numpy as np
import pytest

from luma_gb300 import _abi as A
from luma_gb300 import case as hostcase
from oracle import oracle as O
from tests.golden import cases as CASES
from tests.golden import runner as R


@pytest.mark.parametrize("name", sorted(CASES.CASES))
def test_host_setup_matches_reference(name):
    """Labels, inlet profile, positions and omega computed by the host set-up
    equal the values the reference computed at initialisation."""
    fx = R.fixture(name)
    l0 = R.hierarchy(name)[0]
    assert np.array_equal(l0.typ, fx["typ"])
    assert np.array_equal(l0.ux_in, fx["ux_in"])
    assert np.array_equal(l0.ypos, fx["ypos"])
    assert l0.omega == float(fx["omega"])
    f0, *_ = R.initial_state(l0)
    assert R.sha(f0) == str(fx["f0_sha"])


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("regions")))
def test_host_subgrid_setup_matches_reference(name):
    """Sub-grid labels, coarse limits, positions, inlet profile and omega of
    every refined level, and the parent relabelling, equal the reference's."""
    fx = R.fixture(name)
    levels = R.hierarchy(name)
    assert np.array_equal(levels[0].typ, fx["typ"])
    for lv in levels[1:]:
        k = R.grid_key(lv)
        assert np.array_equal(lv.typ, fx[f"{k}_typ"]), k
        assert lv.omega == float(fx[f"{k}_omega"]), k
        assert tuple(lv.coarse_lims) == tuple(int(x) for x in fx[f"{k}_coarse_lims"]), k
        assert np.array_equal(lv.xpos, fx[f"{k}_xpos"]) and np.array_equal(lv.ypos, fx[f"{k}_ypos"]), k
        assert np.array_equal(lv.ux_in, fx[f"{k}_ux_in"]), k
        f0, *_ = R.initial_state(lv)
        assert R.sha(f0) == str(fx[f"{k}_f0_sha"]), k


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES
                                        if not CASES.CASES[n].get("bodies") and not CASES.CASES[n].get("filaments")))
def test_oracle_bit_exact_vs_reference(name):
    """The restatement reproduces the reference bit for bit (FP64, same
    operation order, no contraction) at every stored step, on every grid."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    grids, levels = R.build_backend(name, lambda d, p: O.OracleGrid(d, p))
    done = 0
    for s in spec["steps"]:
        grids[0].step(s - done)
        done = s
        for g, lv in zip(grids, levels):
            key = R.grid_key(lv)
            st = g.download()
            u, rho, u_sha, rho_sha, f_sha = R.fields_at(fx, key, s, name)
            if u is not None:
                assert np.array_equal(st["u"], u), f"{key} u differs at step {s}"
                assert np.array_equal(st["rho"], rho), f"{key} rho differs at step {s}"
            assert R.sha(st["u"]) == u_sha, f"{key} u differs at step {s}"
            assert R.sha(st["rho"]) == rho_sha, f"{key} rho differs at step {s}"
            assert R.sha(st["f"]) == f_sha, f"{key} f differs at step {s}"
            if key == "L0R0" and f"f_{s}" in fx:
                assert np.array_equal(st["f"], fx[f"f_{s}"])


def test_known_answer_equilibrium_d2q9():
    """The reference test suite's t=0 D2Q9 equilibrium row (rho=1, u=(0.04,0),
    8 decimals) from both the host equilibrium and the oracle."""
    with open(os.path.join(R.HERE, "kat_feq_d2q9.json")) as fp:
        kat = json.load(fp)
    rho = np.array([kat["rho"]])
    u = np.array([kat["u"]])
    feq = hostcase.equilibrium(2, 9, rho, u)[0]
    assert np.allclose(feq, kat["f"], atol=0.5e-8, rtol=0)
    d = hostcase.build_level0(hostcase.Definitions(dims=2, resolution=4, bx=1, by=1))
    g = O.OracleGrid(d.desc())
    n = d.ncell
    f = g.equilibrium(np.tile(u, (n, 1)).reshape(-1), np.full(n, kat["rho"]))
    assert np.allclose(f.reshape(n, 9), np.array(kat["f"])[None, :], atol=0.5e-8, rtol=0)


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("bodies")))
def test_oracle_ibm_bit_exact_vs_reference(name):
    """IBM restatement against the reference: support lists and delta values,
    marker spacing ds, epsilon (same LU as the reference's oracle build),
    marker forces and the flow field at every stored step."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    grids, levels = R.build_backend(name, lambda d, p: O.OracleGrid(d, p))
    ibm = O.OracleIBM()
    for lev, reg, pos in CASES.bodies(name):
        ibm.add_body(grids[lev], pos)
    ibm.initialise()
    mk = ibm.markers(0)
    ref0 = fx["markers_0"]
    assert np.array_equal(mk[:, 7], ref0[:, 9]), "ds"
    assert np.array_equal(mk[:, 6], ref0[:, 8]), "epsilon"
    assert np.array_equal(mk[:, 8], ref0[:, 14]), "support counts"
    sup = ibm.supports(0)
    assert np.array_equal(sup[:, 1:4], fx["supports"][:, 3:6])
    assert np.array_equal(sup[:, 4], fx["supports"][:, 6])
    done = 0
    D = levels[0].defs.dims
    for s in spec["steps"]:
        grids[0].step(s - done)
        done = s
        st = grids[0].download()
        assert np.array_equal(st["u"], fx[f"u_{s}"]) and np.array_equal(st["rho"], fx[f"rho_{s}"])
        assert R.sha(st["f"]) == str(fx[f"f_sha_{s}"])
        for g, lv in zip(grids[1:], levels[1:]):   # refined levels (bodies on a sub-grid)
            key = R.grid_key(lv)
            st = g.download()
            _, _, u_sha, rho_sha, f_sha = R.fields_at(fx, key, s, name)
            assert (R.sha(st["u"]), R.sha(st["rho"]), R.sha(st["f"])) == (u_sha, rho_sha, f_sha), (key, s)
        mk = ibm.markers(0)
        assert np.array_equal(mk[:, 3:3 + D], fx[f"markers_{s}"][:, 5:5 + D]), f"marker force at step {s}"


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("filaments")))
def test_oracle_fem_fsi_bit_exact_vs_reference(name):
    """Flexible filament (co-rotational FEM beam, Newmark/Newton-Raphson,
    FSI sub-iterations) built as the reference's FILAMENT_ARRAY reader builds
    it: marker positions, forces, epsilon and the flow field match the
    reference bit for bit."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    grids, levels = R.build_backend(name, lambda d, p: O.OracleGrid(d, p))
    ibm = O.OracleIBM()
    R.attach_filaments(name, grids, levels, lambda g, **k: ibm.add_filament(g, **k))
    ibm.initialise()
    mk = ibm.markers(0)
    assert np.array_equal(mk[:, 0:3], fx["markers_0"][:, 2:5])
    assert np.array_equal(mk[:, 6], fx["markers_0"][:, 8])
    done = 0
    for s in spec["steps"]:
        grids[0].step(s - done)
        done = s
        st = grids[0].download()
        mk = ibm.markers(0)
        rm = fx[f"markers_{s}"]
        assert np.array_equal(st["u"], fx[f"u_{s}"]) and np.array_equal(st["rho"], fx[f"rho_{s}"])
        assert np.array_equal(mk[:, 0:2], rm[:, 2:4]), "marker positions"
        assert np.array_equal(mk[:, 3:5], rm[:, 5:7]), "marker forces"
        assert np.array_equal(mk[:, 6], rm[:, 8]), "epsilon"


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("bfl")))
def test_bfl_setup_and_oracle_forces_bit_exact_vs_reference(name):
    """The host BFL set-up (circle prefab, labels, surface closure, link
    distances, per-site marker lookup) equals the reference's BFLBody, and the
    restated BFL stream's per-marker momentum-exchange forces equal the
    reference's computeLiftDrag(v, id, g, markerID) at every stored step."""
    fx = R.fixture(name)
    l0 = R.level0(name)
    assert np.array_equal(l0.typ, fx["typ"])
    assert np.array_equal(l0.bfl.site_marker, fx["bfl_site_marker"])
    assert np.array_equal(l0.bfl.q, fx["bfl_q"])
    grids, _ = R.build_backend(name, lambda d, p: O.OracleGrid(d, p))
    done = 0
    for s, ref in zip(fx["bfl_force_steps"], fx["bfl_forces"]):
        grids[0].step(int(s) - done)
        done = int(s)
        assert np.array_equal(grids[0].bfl_forces(), ref), f"marker forces at step {s}"


@pytest.mark.parametrize("name", sorted(n for n in CASES.CASES if CASES.CASES[n].get("store_tav")))
def test_oracle_time_averages_bit_exact_vs_reference(name):
    """Running means of rho, u_p and u_p u_q (_LBM_macro_opt :895-917; IB
    support sites re-averaged once per marker by ibm_updateMacroscopic) equal
    the reference's on every grid at every stored step."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    grids, levels = R.build_backend(name, lambda d, p: O.OracleGrid(d, p))
    if spec.get("bodies"):
        ibm = O.OracleIBM()
        for lev, reg, pos in CASES.bodies(name):
            ibm.add_body(grids[lev], pos)
        ibm.initialise()
    done = 0
    for s in spec["steps"]:
        grids[0].step(s - done)
        done = s
        for g, lv in zip(grids, levels):
            pre = "" if R.grid_key(lv) == "L0R0" else R.grid_key(lv) + "_"
            ta = g.time_averages()
            assert np.array_equal(ta["rho"], fx[f"{pre}rho_ta_{s}"]), (pre, s)
            assert np.array_equal(ta["u"], fx[f"{pre}ui_ta_{s}"]), (pre, s)
            assert np.array_equal(ta["uu"], fx[f"{pre}uiuj_ta_{s}"]), (pre, s)


def test_oracle_momentum_exchange_bit_exact_vs_reference():
    """computeLiftDrag over the solid sites (the Poiseuille channel's walls),
    restated in the oracle: bit-exact with the reference build's force for
    every step (the reference accumulates it during step s from the state
    after step s-1)."""
    ref = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "momex_d2q9.json")))
    oo, _ = R.build_backend(ref["like"], lambda d, p: O.OracleGrid(d, p))
    for s in range(1, ref["steps"] + 1):
        got = oo[0].momex_force()
        assert got.tolist() == ref["forces"][str(s)], (s, got, ref["forces"][str(s)])
        oo[0].step(1)


@pytest.mark.parametrize("n", [1, 5, 33, 64, 96])
def test_oracle_dense_solver_against_scipy(n):
    """The dense LU the oracle (and the device) uses for the epsilon and FEM
    systems, in place of the reference's unpinned LAPACK: residual
    ||Ax - b|| / ||b|| <= 1e-13 and agreement with scipy.linalg's LU
    (lu_factor/lu_solve, a second oracle) within 1e-12, on seeded matrices
    shaped like the epsilon system (diagonally dominant, positive) and on
    general well-conditioned ones."""
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.Generator(np.random.PCG64(20261204 + n))
    for kind in ("epsilon", "general"):
        if kind == "epsilon":
            M = rng.uniform(0.0, 0.3, size=(n, n)) + np.eye(n) * (1.0 + 0.3 * n)
        else:
            M = rng.normal(size=(n, n)) + np.eye(n) * 4.0 * np.sqrt(n)
        b = rng.normal(size=n)
        x = O.lu_solve(M, b)
        assert np.linalg.norm(M @ x - b) <= 1e-13 * np.linalg.norm(b) * max(1.0, np.linalg.cond(M) / 1e2)
        xs = scipy_linalg.lu_solve(scipy_linalg.lu_factor(M), b)
        assert np.max(np.abs(x - xs)) <= 1e-12 * np.max(np.abs(xs)), kind


def test_bfl_builder_large_circle_with_projection_reset():
    """The circle set-up with the closure's projection count reset per
    closure (the bench workload's option: the reference's own count doubles
    per closure marker and never finishes a circle this size): every eBFL
    site has a marker, every marker's voxel is eBFL, link distances lie in
    [0, 1] or are -1, and the labelled ring is closed (every eBFL site has
    an eBFL site among its 4 axis neighbours)."""
    from luma_gb300 import bfl
    d = hostcase.Definitions(dims=2, resolution=128, timestep=1.0 / 3200.0, bx=2.0, by=1.0, re=100, ux0=1.0,
                             walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    l0 = hostcase.build_level0(d)
    body = bfl.circle_body(l0, (0.5, 0.5, 0.0), 0.25, reset_projection=True)
    typ = body.typ.reshape(l0.N, l0.M)
    sm = body.site_marker.reshape(l0.N, l0.M)
    assert np.array_equal(typ == A.BFL, sm >= 0)
    q = body.q
    assert np.all((q == -1.0) | ((q >= 0.0) & (q <= 1.0)))
    assert (q >= 0).sum() > 0
    for i, j in np.argwhere(typ == A.BFL):
        nb = [typ[i + di, j + dj] == A.BFL for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1))]
        assert any(nb), (i, j)


@pytest.mark.parametrize("Q,dims", [(9, 2), (19, 3), (27, 3)])
def test_lattice_tables_known_answers(Q, dims):
    """Lattice tables (src/stdafx.cpp:29-153, src/GridUtils.cpp:31-69):
    opposites negate c, reflections negate one component, the weights'
    moments are 1, 0 and cs^2 I (cs^2 = 1/3), and the host set-up's tables
    are the oracle's."""
    L = O.lattice(Q)
    c, w, opp, refl = L["c"], L["w"], L["opp"], L["refl"]
    for v in range(Q):
        assert np.array_equal(c[opp[v]], -c[v])
        for p in range(dims):
            want = c[v].copy()
            want[p] = -want[p]
            assert np.array_equal(c[refl[p, v]], want), (p, v)
    assert abs(w.sum() - 1.0) <= 1e-15
    assert np.all(np.abs(w @ c) <= 1e-16)
    second = np.einsum("v,va,vb->ab", w, c.astype(float), c.astype(float))
    assert np.allclose(second[:dims, :dims], np.eye(dims) / 3.0, rtol=0, atol=1e-15)
    hc, hw = hostcase.lattice(dims, Q)
    assert np.array_equal(np.asarray(hc), c) and np.array_equal(np.asarray(hw), w)


def test_delta_kernel_known_answers():
    """Roma et al. 3-point kernel (ibm_deltaKernel): value 2/3 at 0, support
    |r| <= 1.5, symmetric, and for any offset the integer shifts sum to 1
    (partition of unity), have zero first moment and squares summing to 1/2;
    the dilation scales the argument."""
    assert O.delta(0.0) == pytest.approx(2.0 / 3.0, abs=1e-16)
    assert O.delta(1.5) == 0.0 and O.delta(1.6) == 0.0
    for r in np.linspace(-0.5, 0.5, 101):
        vals = np.array([O.delta(r - j) for j in range(-3, 4)])
        shifts = r - np.arange(-3, 4)
        assert abs(vals.sum() - 1.0) <= 1e-14, r
        assert abs((shifts * vals).sum()) <= 1e-14, r
        assert abs((vals ** 2).sum() - 0.5) <= 1e-14, r
        assert O.delta(r) == O.delta(-r)
    assert O.delta(0.6, 2.0) == O.delta(0.3, 1.0)


@pytest.mark.parametrize("Q,dims", [(9, 2), (19, 3), (27, 3)])
def test_guo_forcing_moments(Q, dims):
    """Guo forcing of one site (_LBM_forceGrid_opt): no mass source and a
    momentum source of (1 - omega/2) F."""
    rng = np.random.Generator(np.random.PCG64(7 + Q))
    L = O.lattice(Q)
    for omega in (0.8, 1.5, 1.9):
        u = rng.uniform(-0.05, 0.05, size=dims)
        F = rng.uniform(-1e-3, 1e-3, size=dims)
        Fi = O.guo(Q, dims, omega, u, F)
        assert abs(Fi.sum()) <= 1e-18
        mom = Fi @ L["c"][:, :dims].astype(float)
        assert np.allclose(mom, (1.0 - 0.5 * omega) * F, rtol=1e-13, atol=1e-19)


GEOM_DEFS = {
    "geom_d3q19": dict(dims=3, resolution=20, timestep=1.0 / 500.0, bx=2.0, by=1.0, bz=1.0, re=100, ux0=1.0,
                       ibm=True, walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID)),
    "geom_refine_d2q9": dict(dims=2, resolution=40, timestep=1.0 / 800.0, bx=2.0, by=1.0, re=50, ux0=1.0,
                             no_flow=False, ibm=True,
                             walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID)),
}
GEOM_REGIONS = {"geom_refine_d2q9": [((0.5, 0.25, 0.0), (1.0, 0.75, 0.0))]}


@pytest.mark.parametrize("run", [0, 1], ids=["2d", "3d"])
def test_geometry_reader_prefabs_match_reference(run):
    """The geometry reader restatement (circle/sphere, square/cube, plate,
    rigid and flexible filament arrays) gives the reference reader's IB
    bodies: every marker's position, epsilon and ds after initialisation
    equal the reference's (tests/golden/make_geometry.py)."""
    import json
    from luma_gb300 import geometry
    ref = json.load(open(os.path.join(R.HERE, "geometry_prefab.json")))["runs"][run]
    name = ref["case"]
    if name in CASES.CASES:
        l0 = R.level0(name)
    else:
        l0 = hostcase.build_level0(hostcase.Definitions(**GEOM_DEFS[name]))
    bodies = geometry.read_geometry(ref["config"], {(0, 0): l0})
    g = O.OracleGrid(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    ibm = O.OracleIBM()
    for b in bodies:
        if b["kind"] == "ibm":
            ibm.add_body(g, b["positions"])
        else:
            ibm.add_filament(g, **b["args"])
    ibm.initialise()
    got = []
    for ib in range(len(bodies)):
        mk = ibm.markers(ib)
        got += [[ib, m, *mk[m, 0:3], mk[m, 6], mk[m, 7]] for m in range(mk.shape[0])]
    want = ref["markers"]
    assert len(got) == len(want)
    for gr, w in zip(got, want):
        assert gr[:2] == w[:2] and all(float(a) == float(b) for a, b in zip(gr[2:], w[2:])), (gr, w)


def test_geometry_reader_bfl_entries():
    """CIRCLE_SPHERE BFL entries build the BFL bodies of the BFL cases
    (the set-up pinned to the reference's BFLBody above)."""
    from luma_gb300 import geometry
    for name in ("bfl_cyl_d2q9", "bfl_sphere_d3q19"):
        l0 = R.level0(name)
        fx = R.fixture(name)
        base = hostcase.build_level0(CASES.CASES[name]["defs"])
        (b,) = geometry.read_geometry(CASES.geometry_config(name), {(0, 0): base})
        assert b["kind"] == "bfl"
        assert np.array_equal(b["body"].typ, fx["typ"]) and np.array_equal(b["body"].q, fx["bfl_q"])
        assert np.array_equal(b["body"].site_marker, l0.bfl.site_marker)


@pytest.mark.parametrize("run", ["ibm_bbb_2d", "bfl_2d", "ibm_bbb_3d", "bfl_3d", "levels_2d"])
def test_geometry_reader_clouds_match_reference(run):
    """FROM_FILE point clouds (IBM, BFL, BBB; seeded clouds partly off the
    grid, CENTRE and START references, on level 0 and on a refined level)
    give the reference reader's labels, velocity and density on every grid,
    IB markers (position, epsilon, ds after initialisation) and BFL Q table
    and site lookup (tests/golden/make_geometry.py)."""
    from luma_gb300 import geometry
    z = np.load(os.path.join(R.HERE, "geometry_cloud.npz"))
    clouds = {k.split("/", 1)[1]: str(z[k]) for k in z.files if k.startswith("cloud/")}
    name, config = str(z[run + "/case"]), str(z[run + "/config"])
    if name in CASES.CASES:
        grids = [hostcase.build_level0(CASES.CASES[name]["defs"])]
    else:
        grids = [hostcase.build_level0(hostcase.Definitions(**GEOM_DEFS[name]))]
    for r in GEOM_REGIONS.get(name, []):
        grids.append(hostcase.build_subgrid(grids[-1], r[0], r[1]))
    levels = {(g.level, g.region): g for g in grids}
    states = [R.initial_state(g) for g in grids]  # the populations predate the reader
    bodies = geometry.read_geometry(config, levels, clouds=clouds)
    for b in bodies:
        if b["kind"] == "bbb":
            geometry.apply_bbb(levels[(b["level"], b["region"])], b)
    typ = {k: g.typ for k, g in levels.items()}
    for b in bodies:
        if b["kind"] == "bfl":
            typ[(b["level"], b["region"])] = b["body"].typ.reshape(-1)
            assert np.array_equal(b["body"].q, z[run + "/bfl_q"])
            assert np.array_equal(b["body"].site_marker, z[run + "/bfl_marker"])
    keys = sorted({k.split("/")[1] for k in z.files if k.startswith(run + "/L")})
    assert keys == sorted(f"L{lv}R{rg}" for lv, rg in levels)
    for (lv, rg), g in levels.items():
        key = f"{run}/L{lv}R{rg}/"
        assert np.array_equal(typ[(lv, rg)], z[key + "typ"]), (lv, rg)
        assert np.array_equal(g.u, z[key + "u"]) and np.array_equal(g.rho, z[key + "rho"]), (lv, rg)
    ibs = [b for b in bodies if b["kind"] == "ibm"]
    assert bool(ibs) == (run + "/markers" in z.files)
    if ibs:
        og = {}
        for g, st in zip(grids, states):
            og[(g.level, g.region)] = O.OracleGrid(g.desc(), og.get((g.level - 1, 0)))
            og[(g.level, g.region)].upload(*st, t=0)
        ibm = O.OracleIBM()
        for b in ibs:
            ibm.add_body(og[(b["level"], b["region"])], b["positions"])
        ibm.initialise()
        got = []
        for ib in range(len(ibs)):
            mk = ibm.markers(ib)
            got += [[ib, m, *mk[m, 0:3], mk[m, 6], mk[m, 7]] for m in range(mk.shape[0])]
        assert np.array_equal(np.array(got), z[run + "/markers"])


def test_cloud_reader_quirks():
    """io_readInCloud's stream reading: a line without values (the one after
    a final newline) repeats the previous point, a missing z keeps the
    previous z; std::round rounds halves away from zero."""
    from luma_gb300 import geometry
    pts = geometry.read_cloud("1 2 3\n4 5\n", 3)
    assert pts == [(1.0, 2.0, 3.0), (4.0, 5.0, 3.0), (4.0, 5.0, 3.0)]
    assert geometry.read_cloud("1 2 3\n4 5", 2) == [(1.0, 2.0, 0.0), (4.0, 5.0, 0.0)]
    with pytest.raises(ValueError):
        geometry.read_cloud("\n1 2 3", 3)
    assert [geometry._cround(v) for v in (0.5, 1.5, 2.5, -0.5, -2.5, 2.4999)] == [1, 2, 3, -1, -3, 2]


INITVEL_DEFS = {
    "initvel_d2q9": dict(dims=2, resolution=20, timestep=1.0 / 400.0, bx=2.0, by=1.0, re=50, ux0=1.0,
                         no_flow=False,
                         walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID)),
    "initvel_d3q19": dict(dims=3, resolution=4, timestep=1.0 / 80.0, bx=3.0, by=2.0, bz=1.5, re=10, ux0=0.0,
                          no_flow=False),
}


@pytest.mark.parametrize("name", sorted(INITVEL_DEFS))
def test_initial_velocity_file_matches_reference(name):
    """L_INIT_VELOCITY_FROM_FILE: the level-0 velocity and populations the
    reference starts from, for shuffled seeded files with duplicates, points
    off the grid, more points than sites and (3D) a short line that freezes
    every later value (tests/golden/make_initvel.py)."""
    z = np.load(os.path.join(R.HERE, "initial_velocity.npz"))
    d = hostcase.Definitions(**INITVEL_DEFS[name])
    l0 = hostcase.build_level0(d)
    u = hostcase.initial_velocity_from_file(str(z[name + "/text"]), l0)
    assert np.array_equal(u, z[name + "/u"])
    f = hostcase.equilibrium(d.dims, d.Q, l0.rho, u).reshape(-1)
    assert np.array_equal(f, z[name + "/f"])
    with pytest.raises(ValueError):
        hostcase.initial_velocity_from_file("\n".join(str(z[name + "/text"]).split("\n")[:100]), l0)


def test_velocity_stream_reader_semantics():
    """The stream rules the initial-velocity reader relies on: a missing
    value keeps the variable, a non-number stores 0, and after either every
    later extraction fails."""
    rd = hostcase._StreamReader()
    rd.reset("1.5 2e1 -.25")
    assert [rd.extract() for _ in range(3)] == [1.5, 20.0, -0.25]
    assert rd.extract() == -0.25 and rd.failed
    rd.reset("7 8 9")
    assert rd.extract() == -0.25
    rd = hostcase._StreamReader()
    rd.reset("3 abc 4")
    assert [rd.extract(), rd.extract(), rd.extract()] == [3.0, 0.0, 0.0]
    rd = hostcase._StreamReader()
    rd.reset("1e+ 5")
    assert rd.extract() == 0.0 and rd.failed


def test_inlet_profile_file_matches_reference():
    """L_USE_INLET_PROFILE on a refined channel: every grid's inlet profile,
    initial velocity and populations equal the reference's, including the
    point a final newline appends (its y is the last value read), which
    sets the top rows by extrapolation (tests/golden/make_initvel.py)."""
    z = np.load(os.path.join(R.HERE, "initial_velocity.npz"))
    case = "inletfile_refine_d2q9"
    d = hostcase.Definitions(dims=2, resolution=40, timestep=1.0 / 800.0, bx=2.0, by=1.0, re=50, ux0=1.0,
                             no_flow=False, inlet_profile=str(z[case + "/text"]),
                             walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    g0 = hostcase.build_level0(d)
    g1 = hostcase.build_subgrid(g0, (0.5, 0.25, 0.0), (1.0, 0.75, 0.0))
    for g, key in ((g0, "L0R0"), (g1, "L1R0")):
        assert np.array_equal(g.ux_in, z[f"{case}/{key}/uxin"]), key
        assert np.array_equal(g.u, z[f"{case}/{key}/u"]), key
        f = hostcase.equilibrium(2, 9, g.rho, g.u).reshape(-1)
        assert np.array_equal(f, z[f"{case}/{key}/f"]), key
    with pytest.raises(ValueError):
        hostcase.inlet_profile_from_file("0 0.5 0 0.1 0 0", g0.ypos)


def test_universal_epsilon_matches_reference():
    """L_UNIVERSAL_EPSILON_CALC: one epsilon system over two circles whose
    supports overlap and a square.  The oracle and the library's host set-up
    (luma_ibm_setup_host, what luma_gpu_ibm_initialise runs for rigid bodies)
    give the reference's epsilon and ds bit for bit; per-body systems do not
    (tests/golden/make_geometry.py, oracle/cases/ibm_universal_d2q9.h)."""
    import ctypes as C
    import json
    from luma_gb300 import geometry
    ref = json.load(open(os.path.join(R.HERE, "geometry_prefab.json")))["runs"][2]
    assert ref["case"] == "ibm_universal_d2q9"
    defs = hostcase.Definitions(dims=2, resolution=40, timestep=1.0 / 1000.0, bx=2.0, by=1.0, re=100, ux0=1.0,
                                ibm=True, universal_epsilon=True,
                                walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    l0 = hostcase.build_level0(defs)
    assert l0.desc().flags & A.FLAG_UNIVERSAL_EPSILON
    bodies = geometry.read_geometry(ref["config"], {(0, 0): l0})
    want = np.array(ref["markers"])
    oracle_eps = {}
    for universal in (True, False):
        g = O.OracleGrid(l0.desc())
        g.upload(*R.initial_state(l0), t=0)
        ibm = O.OracleIBM()
        for b in bodies:
            ibm.add_body(g, b["positions"])
        ibm.initialise(universal=universal)
        got = np.array([[ib, m, *mk[m, 0:3], mk[m, 6], mk[m, 7]]
                        for ib in range(len(bodies)) for mk in [ibm.markers(ib)] for m in range(mk.shape[0])])
        assert np.array_equal(got, want) == universal
        oracle_eps[universal] = got[:, 5]
    lib_path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "luma_gb300", "_build",
                            "libluma_gpu.so")
    if not os.path.exists(lib_path):
        from luma_gb300 import build
        build.build()
    try:
        lib = C.CDLL(lib_path)
    except OSError as e:
        pytest.skip(f"cannot load CUDA library here: {e}")
    dp = C.POINTER(C.c_double)
    lib.luma_ibm_setup_host.argtypes = [C.POINTER(A.GridDesc), C.c_int, C.POINTER(C.c_int), dp, C.c_int, dp, dp,
                                        C.POINTER(C.c_int)]
    d = l0.desc()
    nm = np.array([len(b["positions"]) for b in bodies], dtype=np.int32)
    pos = np.ascontiguousarray(np.concatenate([np.asarray(b["positions"], float).reshape(-1, 3) for b in bodies]))
    for universal in (1, 0):
        eps, ds = np.zeros(nm.sum()), np.zeros(nm.sum())
        ns = np.zeros(nm.sum(), dtype=np.int32)
        assert lib.luma_ibm_setup_host(C.byref(d), len(nm), nm.ctypes.data_as(C.POINTER(C.c_int)),
                                       pos.ctypes.data_as(dp), universal, eps.ctypes.data_as(dp),
                                       ds.ctypes.data_as(dp), ns.ctypes.data_as(C.POINTER(C.c_int))) == 0
        assert np.array_equal(ds, want[:, 6])
        assert np.array_equal(eps, want[:, 5]) == bool(universal)
        assert np.array_equal(eps, oracle_eps[bool(universal)])


def test_universal_epsilon_refused_with_flexible_bodies():
    """With a flexible filament on the grid the reference re-solves the
    coupled system every FSI sub-iteration; the oracle refuses the universal
    mode there instead of solving something else."""
    import json
    from luma_gb300 import geometry
    ref = json.load(open(os.path.join(R.HERE, "geometry_prefab.json")))["runs"][0]
    l0 = R.level0(ref["case"])
    bodies = geometry.read_geometry(ref["config"], {(0, 0): l0})
    g = O.OracleGrid(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    ibm = O.OracleIBM()
    for b in bodies:
        if b["kind"] == "ibm":
            ibm.add_body(g, b["positions"])
        else:
            ibm.add_filament(g, **b["args"])
    with pytest.raises(RuntimeError, match="flexible"):
        ibm.initialise(universal=True)
        assert ns.min() >= 4


def test_subgrid_edges_round_half_away_from_zero():
    """Refined-region limits on half coarse cells: the edges follow
    std::round (halves away from zero), so the refined grid's size, site
    positions and both grids' labels equal the reference's
    (oracle/cases/refine_halfcell_d2q9.h, tests/golden/make_initvel.py);
    round-half-to-even would give a 12 x 8 grid shifted by a coarse cell."""
    z = np.load(os.path.join(R.HERE, "initial_velocity.npz"))
    d = hostcase.Definitions(dims=2, resolution=4, timestep=1.0 / 80.0, bx=4.0, by=2.0, re=50, ux0=1.0,
                             walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    g0 = hostcase.build_level0(d)
    g1 = hostcase.build_subgrid(g0, (0.625, 0.375, 0.0), (2.125, 1.625, 0.0))
    case = "refine_halfcell_d2q9"
    for g, key in ((g0, "L0R0"), (g1, "L1R0")):
        assert np.array_equal(g.typ, z[f"{case}/{key}/typ"]), key
        assert np.array_equal(g.xpos, z[f"{case}/{key}/xpos"]), key
        assert np.array_equal(g.ypos, z[f"{case}/{key}/ypos"]), key
    assert (g1.N, g1.M) == (12, 10)
