"""L_UNIVERSAL_EPSILON_CALC stepped on the device.

The reference, built with L_UNIVERSAL_EPSILON_CALC, solves one epsilon
system over every rigid body of a level (ObjectManager::ibm_findEpsilon,
src/ObjectManager_ops_ibm.cpp:773-920, :1067-1142) instead of one per body;
bodies whose supports overlap then couple.  The case is the geometry
reader's two overlapping circles and a square on a D2Q9 channel (the case
whose set-up tests/test_oracle_golden.py pins bit for bit against the
reference build).  Here the GPU grid created with LUMA_FLAG_UNIVERSAL_EPSILON
steps against the oracle's universal mode: epsilon, ds and support counts
equal, then after 400 steps FP64 fields within rel L2 1e-10 and marker forces
within 1e-9; shifted FP32 within its bounds (u rel L2 2e-4, forces 1e-3).
The flow starts uniform: over the first few dozen steps some bodies' marker
forces are residuals of order 1e-9 (against 1e-6 on the others) whose
relative value moves by 1e-7 when the initial state moves by 1e-15 in the
oracle itself; by step 400 every body carries a developed force (3.5e-3 to
6e-3) and that sensitivity is 2e-13.
"""
import json
import os

import numpy as np
import pytest

from luma_gb300 import _abi as A
from luma_gb300 import case as hostcase
from luma_gb300 import geometry
from oracle import oracle as O
from tests.golden import runner as R

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


def _universal_case():
    ref = json.load(open(os.path.join(R.HERE, "geometry_prefab.json")))["runs"][2]
    assert ref["case"] == "ibm_universal_d2q9"
    defs = hostcase.Definitions(dims=2, resolution=40, timestep=1.0 / 1000.0, bx=2.0, by=1.0, re=100, ux0=1.0,
                                ibm=True, universal_epsilon=True,
                                walls=(A.VELOCITY, A.EXTRAPOLATE_RIGHT, A.SOLID, A.SOLID, A.FLUID, A.FLUID))
    l0 = hostcase.build_level0(defs)
    bodies = geometry.read_geometry(ref["config"], {(0, 0): l0})
    return l0, [b["positions"] for b in bodies if b["kind"] == "ibm"]


@pytest.mark.parametrize("prec", [A.PREC_FP64, A.PREC_FP32_SHIFTED], ids=["fp64", "fp32s"])
def test_universal_epsilon_steps_match_oracle(prec):
    from luma_gb300.gpu import GpuGrid
    l0, bodies = _universal_case()
    assert len(bodies) == 3
    desc = l0.desc(precision=prec)
    assert desc.flags & A.FLAG_UNIVERSAL_EPSILON
    g = GpuGrid(desc)
    o = O.OracleGrid(l0.desc())
    state = R.initial_state(l0)
    g.upload(*state, t=0)
    o.upload(*state, t=0)
    oibm = O.OracleIBM()
    for pos in bodies:
        g.ibm_add_body(pos)
        oibm.add_body(o, pos)
    g.ibm_initialise()
    oibm.initialise(universal=True)
    for b in range(len(bodies)):
        gm, om = g.ibm_markers(b), oibm.markers(b)
        assert np.array_equal(gm[:, 6:9], om[:, 6:9]), b   # epsilon, ds, supports
    g.step(400)
    o.step(400)
    gs, os_ = g.download(), o.download()
    eu = rel_l2(gs["u"], os_["u"])
    for b in range(len(bodies)):
        gm, om = g.ibm_markers(b), oibm.markers(b)
        ef = rel_l2(gm[:, 3:5], om[:, 3:5])
        if prec == A.PREC_FP64:
            assert ef <= 1e-9, (b, ef)
        else:
            assert ef <= 1e-3, (b, ef)
    if prec == A.PREC_FP64:
        assert eu <= 1e-10 and rel_l2(gs["f"], os_["f"]) <= 1e-10, eu
    else:
        assert eu <= 2e-4, eu
