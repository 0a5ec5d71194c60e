"""The LUMA-side shim (luma_gb300/shim/gridobj_gpu.cpp) built into the
reference itself.

oracle/build_ref.py compiles the reference's own sources with the shim and
the harness twice per case: linked with libluma_gpu.so (the drop-in as a
maintainer builds it; that the link succeeds shows every entry point the
shim calls is in the library) and linked with the oracle behind the same
entry points (oracle/abi_on_oracle.c).  The second runs here: the
reference's initialisation (grids, labels, sub-grids, geometry, IB bodies),
then every step through the shim — GridObj tree to descriptors, state up,
LBM_multi_opt across the ABI, state back into the GridObj members — and its
dumps must equal, byte for byte, those of the same reference build stepping
with its own GridObj::LBM_multi_opt.  The device side of each ABI call is
pinned by the GPU tests; the reference sources are not on the GPU machines,
so the GPU-linked build is not run there.
"""
import filecmp
import os
import subprocess

import numpy as np
import pytest

from oracle import build_ref
from tests.golden import cases as CASES

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(build_ref.DEFAULT_REF, "src")),
                                reason="reference checkout not present")

SHIM_CASES = [("refine_d2q9", 30), ("poiseuille_d2q9", 60), ("ibm_cyl_d2q9", 20), ("tgv_d3q19", 6),
              ("ibm_sphere_refine_d3q19", 4), ("kbc_d3q27", 4)]


def _inputs(name, work):
    args = []
    init = CASES.initial_fields(name)
    if init is not None:
        p = os.path.join(work, "init_u.bin")
        init["u"].astype(np.float64).tofile(p)
        args += ["--init-u", p]
    blist = CASES.bodies(name)
    if blist:
        p = os.path.join(work, "markers.in")
        CASES.write_marker_file(p, blist)
        args += ["--markers", p]
    return args


def test_shim_links_against_the_gpu_library():
    exe = build_ref.build_case("refine_d2q9", shim="gpu")
    assert os.path.exists(exe)


@pytest.mark.parametrize("name,steps", SHIM_CASES, ids=[n for n, _ in SHIM_CASES])
def test_shim_reproduces_reference_step(name, steps, tmp_path):
    plain = build_ref.build_case(name)
    shim = build_ref.build_case(name, shim="oracle")
    inp = _inputs(name, str(tmp_path))
    common = ["--steps", str(steps), "--dump-every", str(steps)] + inp
    subprocess.run([plain, "--out", str(tmp_path / "plain"), *common], check=True, capture_output=True)
    r = subprocess.run([shim, "--out", str(tmp_path / "shim"), "--gpu-shim", "0", *common],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    a, b = tmp_path / "plain" / f"s{steps}", tmp_path / "shim" / f"s{steps}"
    files = sorted(f for f in os.listdir(a) if f.endswith(".bin") or f == "markers.txt")
    assert any(f.endswith("_f.bin") for f in files)
    match, mismatch, errors = filecmp.cmpfiles(a, b, files, shallow=False)
    assert not mismatch and not errors, (mismatch, errors)
