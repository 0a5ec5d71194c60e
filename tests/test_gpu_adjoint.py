"""Discrete adjoint of the time-averaged drag against central finite
differences of the oracle (the reference's FP64 arithmetic), on a small
D2Q9 channel with a rigid cylinder of 32 markers on perturbed radii.

Bounds: the FP64 forward drag equals the oracle's within 1e-10 (relative);
the FP64 adjoint gradients equal central differences (h = 1e-4 relative for
the inlet scale, 1e-4 lattice units for marker coordinates) within 1e-4 of
the largest difference; the FP32-shifted adjoint is within 1e-3 (inlet) and
1e-2 (markers, max-norm relative) of the FP64 adjoint.
"""
import numpy as np
import pytest

from luma_gb300 import _abi as A
from luma_gb300 import adjoint as ADJ
from oracle import oracle as O

pytestmark = pytest.mark.gpu

T, KCK = 150, 40          # steps, checkpoint interval (ragged last segment)


@pytest.fixture(scope="module")
def small():
    return ADJ.cylinder_channel(nx=100, ny=40, diameter_lu=10.0, n_markers=32, sigma_lu=0.1,
                                timestep=1.0 / 600.0, re=20.0, nsteps=T, checkpoint_every=KCK)


def oracle_drag(c, inlet_scale=1.0, markers=None):
    """J of the case on the oracle: marker forces after every step."""
    l0, f0, u, rho = ADJ.initial_state(c.defs, inlet_scale)
    og = O.OracleGrid(l0.desc())
    og.upload(f0, u, rho, l0.force_xyz.copy(), t=0)
    ib = O.OracleIBM()
    ib.add_body(og, c.markers if markers is None else markers)
    ib.initialise()
    J = 0.0
    for _ in range(c.nsteps):
        og.step(1)
        mk = ib.markers(0)
        J += float(np.sum(mk[:, 3] * mk[:, 6] * mk[:, 7]))
    og.close()
    return J / c.nsteps


@pytest.fixture(scope="module")
def fp64(small):
    return ADJ.drag_and_gradient(small, A.PREC_FP64)


def test_forward_drag_matches_oracle(small, fp64):
    J = fp64[0]
    Jo = oracle_drag(small)
    assert J != 0.0
    assert abs(J - Jo) <= 1e-10 * abs(Jo), (J, Jo)


def test_inlet_gradient_matches_central_differences(small, fp64):
    _, gs, _ = fp64
    h = 1e-4
    fd = (oracle_drag(small, 1.0 + h) - oracle_drag(small, 1.0 - h)) / (2 * h)
    assert abs(gs - fd) <= 1e-4 * abs(fd), (gs, fd)


def test_marker_gradient_matches_central_differences(small, fp64):
    _, _, gx = fp64
    dh = 1.0 / small.defs.resolution
    h = 1e-4 * dh
    picks = [(0, 0), (0, 1), (5, 0), (5, 1), (11, 0), (11, 1), (19, 0), (19, 1), (26, 0), (26, 1)]
    fd = []
    for m, d in picks:
        plus, minus = small.markers.copy(), small.markers.copy()
        plus[m, d] += h
        minus[m, d] -= h
        fd.append((oracle_drag(small, markers=plus) - oracle_drag(small, markers=minus)) / (2 * h))
    fd = np.array(fd)
    ad = np.array([gx[m, d] for m, d in picks])
    scale = np.max(np.abs(fd))
    assert scale > 0
    assert np.max(np.abs(ad - fd)) <= 1e-4 * scale, np.c_[ad, fd]


@pytest.mark.parametrize("every", [T, 75])
def test_checkpoint_interval_does_not_change_the_gradient(small, fp64, every):
    """One segment (captured as a graph) and odd segments (run uncaptured)
    against the ragged 40-step segmentation."""
    one = ADJ.DragCase(small.defs, small.markers, small.nsteps, every)
    J1, gs1, gx1 = ADJ.drag_and_gradient(one, A.PREC_FP64)
    J, gs, gx = fp64
    assert J1 == J
    assert abs(gs1 - gs) <= 1e-12 * abs(gs)
    assert np.max(np.abs(gx1 - gx)) <= 1e-12 * np.max(np.abs(gx))


def test_fp32_shifted_adjoint_close_to_fp64(small, fp64):
    J, gs, gx = fp64
    J32, gs32, gx32 = ADJ.drag_and_gradient(small, A.PREC_FP32_SHIFTED)
    assert abs(J32 - J) <= 1e-4 * abs(J), (J32, J)
    assert abs(gs32 - gs) <= 1e-3 * abs(gs), (gs32, gs)
    assert np.max(np.abs(gx32 - gx)) <= 1e-2 * np.max(np.abs(gx))


def test_backward_restores_forward_state_and_runs_once(small):
    g, _ = ADJ.make_grid(small, A.PREC_FP64)
    try:
        g.adj_forward(small.nsteps, small.checkpoint_every, 0)
        after = g.download()
        t = g.t
        assert g.adj_memory() > 0
        g.adj_backward(1.0)
        back = g.download()
        assert g.t == t
        for k in ("f", "u", "rho"):
            assert np.array_equal(after[k], back[k]), k
        from luma_gb300.gpu import LumaError
        with pytest.raises(LumaError):
            g.adj_backward(1.0)
    finally:
        g.close()


def test_repeated_gradient_on_one_grid(small, fp64):
    """A second forward/backward of the same length on the same grid (state
    and captured segment graphs kept) from the same initial state gives the
    same J and gradients; a different length rebuilds the state."""
    g, l0 = ADJ.make_grid(small, A.PREC_FP64)
    _, f0, u, rho = ADJ.initial_state(small.defs)
    force = l0.force_xyz.copy() if l0.force_xyz is not None else None
    J0, gs0, gx0 = fp64
    try:
        for nsteps in (small.nsteps, small.nsteps, 2 * KCK):
            g.upload(f0, u, rho, force, t=0)
            J = g.adj_forward(nsteps, small.checkpoint_every, 0)
            gs, gx = g.adj_backward(1.0)
            if nsteps == small.nsteps:
                assert J == J0
                assert abs(gs - gs0) <= 1e-12 * abs(gs0)
                assert np.max(np.abs(gx - gx0)) <= 1e-12 * np.max(np.abs(gx0))
        short = ADJ.DragCase(small.defs, small.markers, 2 * KCK, small.checkpoint_every)
        Js, gss, gxs = ADJ.drag_and_gradient(short, A.PREC_FP64)
        assert J == Js
        assert abs(gs - gss) <= 1e-12 * abs(gss)
        assert np.max(np.abs(gx - gxs)) <= 1e-12 * np.max(np.abs(gxs))
    finally:
        g.close()


def test_autograd_function_contract(small, fp64):
    torch = pytest.importorskip("torch")
    fn = ADJ.drag_function()
    s = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    X = torch.tensor(small.markers, dtype=torch.float64, requires_grad=True)
    J = fn.apply(s, X, small, A.PREC_FP64)
    (2.0 * J).backward()
    J0, gs, gx = fp64
    assert float(J.detach()) == J0
    assert abs(float(s.grad) - 2.0 * gs) <= 1e-12 * abs(gs)
    assert np.allclose(X.grad[:, :2].numpy(), 2.0 * gx, rtol=1e-10, atol=1e-12 * np.max(np.abs(gx)))
    assert np.all(X.grad[:, 2].numpy() == 0.0)


def test_scope_is_checked(small):
    from luma_gb300.gpu import LumaError
    g, _ = ADJ.make_grid(small, A.PREC_FP64)
    try:
        with pytest.raises(LumaError):
            g.adj_forward(10, 5, 3)        # no body 3
        with pytest.raises(LumaError):
            g.adj_backward(1.0)            # no forward recorded
    finally:
        g.close()


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED])
def test_adjoint_workload_matches_reference_finite_differences(prec):
    """The 400 x 160 channel, 64-marker cylinder, 4000 steps, checkpoints
    every 100: adjoint gradients (FP64, and FP32-shifted as the workload
    runs) within 1e-4 of central differences of the reference's own build
    (tests/golden/make_adjoint_fd.py); the FP64 drag within 1e-10 of the
    reference's."""
    import json
    import os
    ref = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "adjoint_fd_cyl400.json")))
    c = ADJ.cylinder_channel(nsteps=ref["steps"], checkpoint_every=ref["checkpoint_every"])
    J, gs, gx = ADJ.drag_and_gradient(c, prec)
    if prec == A.PREC_FP64:
        assert abs(J - ref["J"]) <= 1e-10 * abs(ref["J"]), (J, ref["J"])
    else:
        assert abs(J - ref["J"]) <= 1e-4 * abs(ref["J"]), (J, ref["J"])
    assert abs(gs - ref["fd_inlet"]) <= 1e-4 * abs(ref["fd_inlet"]), (gs, ref["fd_inlet"])
    fd = np.array([r["fd"] for r in ref["markers"]])
    ad = np.array([gx[r["marker"], r["dim"]] for r in ref["markers"]])
    assert np.max(np.abs(ad - fd)) <= 1e-4 * np.max(np.abs(fd)), np.c_[ad, fd]
