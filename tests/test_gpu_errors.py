"""Error behaviour of the C ABI on the GPU: every refusal comes back as a
negative status with a message (the reference's L_ERROR exits instead), and
the handle stays usable or is never created."""
import numpy as np
import pytest

from luma_gb300 import _abi as A
from luma_gb300 import case as hc
from tests.golden import runner as R

pytestmark = pytest.mark.gpu


def create(desc, parent=None):
    from luma_gb300.gpu import GpuGrid
    return GpuGrid(desc, parent)


def expect(code, fn, *args, match=None):
    from luma_gb300.gpu import LumaError
    with pytest.raises(LumaError) as ei:
        fn(*args)
    assert ei.value.code == code, (ei.value.code, str(ei.value))
    if match:
        assert match in str(ei.value), str(ei.value)


def channel():
    return R.level0("poiseuille_d2q9")


def test_descriptor_refusals():
    l0 = channel()
    d = l0.desc()
    d.Q = 19
    expect(A.LUMA_E_INVALID, create, d, match="D2Q19")
    d = l0.desc()
    d.omega = 2.5
    expect(A.LUMA_E_INVALID, create, d, match="omega")
    d = l0.desc()
    d.precision = 7
    expect(A.LUMA_E_INVALID, create, d, match="precision")
    t3 = R.level0("tgv_d3q19")
    d = t3.desc()
    d.collision = A.COLL_KBC
    expect(A.LUMA_E_INVALID, create, d, match="D3Q27")


def test_site_label_refusals():
    l0 = channel()
    typ = l0.typ.copy()
    typ[500] = A.BFL
    l0.typ = typ
    g = create(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    expect(A.LUMA_E_STATE, g.step, 1, match="BFL")   # BFL labels without a BFL body
    sm = np.full(l0.ncell, -1, dtype=np.int32)
    expect(A.LUMA_E_INVALID, g.bfl_set, sm, np.full((0, 9), -1.0), match="no marker")
    sm[500] = 3
    expect(A.LUMA_E_INVALID, g.bfl_set, sm, np.full((2, 9), -1.0), match="marker 3")
    l0 = channel()
    typ = l0.typ.reshape(l0.N, l0.M, l0.K).copy()
    typ[1, 10, 0] = A.EXTRAPOLATE_RIGHT
    l0.typ = typ.reshape(-1)
    expect(A.LUMA_E_INVALID, create, l0.desc(), match="i=1")


def test_step_and_state_refusals():
    g = create(channel().desc())
    expect(A.LUMA_E_INVALID, g.step, -1, match="negative")
    levels = R.hierarchy("refine_d2q9")
    root = create(levels[0].desc())
    child = create(levels[1].desc(), root)
    expect(A.LUMA_E_INVALID, child.step, 1, match="level-0")
    # the grids still work after the refusals
    for x, lv in ((root, levels[0]), (child, levels[1])):
        x.upload(*R.initial_state(lv), t=0)
    root.step(2)
    assert root.t == 2 and np.isfinite(root.download()["u"]).all()


def test_ibm_refusals():
    g = create(channel().desc())
    pos = np.array([[0.5, 0.5, 0.0], [0.51, 0.5, 0.0]])
    expect(A.LUMA_E_INVALID, g.ibm_add_body, pos, match="LUMA_FLAG_IBM")
    l0 = R.level0("ibm_cyl_d2q9")
    g = create(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    far = np.array([[50.0, 0.5, 0.0], [50.01, 0.5, 0.0]])
    g.ibm_add_body(far)
    expect(A.LUMA_E_DOMAIN, g.ibm_initialise, match="inside its grid")


def test_adjoint_scope_refusals():
    from luma_gb300 import adjoint as ADJ
    c = ADJ.cylinder_channel(nx=100, ny=40, diameter_lu=10.0, n_markers=32, timestep=1.0 / 600.0, re=20.0,
                             nsteps=20, checkpoint_every=10)
    g, _ = ADJ.make_grid(c, A.PREC_FP64)
    expect(A.LUMA_E_INVALID, g.adj_forward, 0, 10, 0)
    expect(A.LUMA_E_STATE, g.adj_backward, 1.0)
    g.close()
    # a grid without IB bodies
    plain = create(channel().desc())
    expect(A.LUMA_E_STATE, plain.adj_forward, 10, 5, 0)
