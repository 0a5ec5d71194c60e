"""The CPU oracle against the reference's own outputs (golden fixtures made
by tests/golden/make_golden.py from the reference's serial build)."""
import json
import os

import numpy as np
import pytest

from luma_gb300 import case as hostcase
from oracle import oracle as O
from tests.golden import cases as CASES
from tests.golden import runner as R


@pytest.mark.parametrize("name", sorted(CASES.CASES))
def test_host_setup_matches_reference(name):
    """Labels, inlet profile, positions and omega computed by the host set-up
    equal the values the reference computed at initialisation."""
    fx = R.fixture(name)
    l0 = R.level0(name)
    assert np.array_equal(l0.typ, fx["typ"])
    assert np.array_equal(l0.ux_in, fx["ux_in"])
    assert np.array_equal(l0.ypos, fx["ypos"])
    assert l0.omega == float(fx["omega"])
    f0, *_ = R.initial_state(l0)
    assert R.sha(f0) == str(fx["f0_sha"])


@pytest.mark.parametrize("name", sorted(CASES.CASES))
def test_oracle_bit_exact_vs_reference(name):
    """The restatement reproduces the reference bit for bit (FP64, same
    operation order, no contraction) at every stored step."""
    spec = CASES.CASES[name]
    fx = R.fixture(name)
    l0 = R.level0(name)
    g = O.OracleGrid(l0.desc())
    g.upload(*R.initial_state(l0), t=0)
    done = 0
    for s in spec["steps"]:
        g.step(s - done)
        done = s
        st = g.download()
        assert np.array_equal(st["u"], fx[f"u_{s}"]), f"u differs at step {s}"
        assert np.array_equal(st["rho"], fx[f"rho_{s}"]), f"rho differs at step {s}"
        assert R.sha(st["f"]) == str(fx[f"f_sha_{s}"]), f"f differs at step {s}"
        if f"f_{s}" in fx:
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
