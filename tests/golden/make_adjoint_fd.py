"""Central finite differences of the reference's time-averaged drag for the
adjoint workload, from the reference itself.

Builds the reference's own serial code for ``oracle/cases/adjoint_cyl_d2q9.h``
(400 x 160 D2Q9 channel, parabolic inlet of peak 0.05 lu, rigid cylinder of
64 injected markers on seeded perturbed radii; ``luma_gb300.adjoint.
cylinder_channel()`` builds the same case) and runs it for 4000 steps with
``--drag-out``, which writes the time average of body 0's lattice-unit drag
(io_writeLiftDrag's per-marker sum, src/ObjectManager_ops_io.cpp:105-121).
Runs: the base case; the velocity of every inlet site scaled by 1 +- h
(h = 1e-4); and a few marker coordinates moved by +- 1e-4 lattice units.
The runs are independent processes, spread over the host cores.

Output: ``adjoint_fd_cyl400.json`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_adjoint_fd.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py) [--steps 4000]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from luma_gb300 import adjoint as ADJ  # noqa: E402
from oracle import build_ref  # noqa: E402
from tests.golden import cases as CASES  # noqa: E402

CASE = "adjoint_cyl_d2q9"
H_INLET = 1e-4
H_MARKER_LU = 1e-4
PICKS = [(0, 0), (0, 1), (21, 0), (21, 1), (42, 0), (42, 1)]


def run(exe: str, steps: int, inlet_scale: float, markers: np.ndarray) -> float:
    c = ADJ.cylinder_channel(nsteps=steps)
    _, _, u, _ = ADJ.initial_state(c.defs, inlet_scale)
    work = tempfile.mkdtemp(prefix="adjfd_")
    upath = os.path.join(work, "init_u.bin")
    np.asarray(u, dtype=np.float64).tofile(upath)
    mpath = os.path.join(work, "markers.in")
    CASES.write_marker_file(mpath, [(0, 0, markers)])
    dpath = os.path.join(work, "drag.txt")
    subprocess.run([exe, "--out", work, "--steps", str(steps), "--init-u", upath, "--markers", mpath,
                    "--drag-out", dpath], check=True, capture_output=True)
    with open(dpath) as fp:
        J, n = fp.read().split()
    assert int(n) == steps
    return float(J)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    exe = build_ref.build_case(CASE, a.ref)
    c = ADJ.cylinder_channel(nsteps=a.steps)
    dh = 1.0 / c.defs.resolution
    jobs = {"base": (1.0, c.markers), "inlet+": (1.0 + H_INLET, c.markers), "inlet-": (1.0 - H_INLET, c.markers)}
    for m, d in PICKS:
        for sgn, tag in ((1.0, "+"), (-1.0, "-")):
            mk = c.markers.copy()
            mk[m, d] += sgn * H_MARKER_LU * dh
            jobs[f"x{m}_{d}{tag}"] = (1.0, mk)
    with cf.ProcessPoolExecutor(max_workers=a.jobs, mp_context=__import__("multiprocessing").get_context("spawn")) as ex:
        futs = {k: ex.submit(run, exe, a.steps, s, mk) for k, (s, mk) in jobs.items()}
        J = {k: f.result() for k, f in futs.items()}
    out = {
        "case": CASE, "steps": a.steps, "checkpoint_every": c.checkpoint_every, "u_max": ADJ.inlet_u_max(c),
        "h_inlet": H_INLET, "h_marker_lu": H_MARKER_LU, "J": J["base"],
        "J_inlet": [J["inlet+"], J["inlet-"]],
        "fd_inlet": (J["inlet+"] - J["inlet-"]) / (2 * H_INLET),
        "markers": [dict(marker=m, dim=d, J_plus=J[f"x{m}_{d}+"], J_minus=J[f"x{m}_{d}-"],
                         fd=(J[f"x{m}_{d}+"] - J[f"x{m}_{d}-"]) / (2 * H_MARKER_LU * dh)) for m, d in PICKS],
    }
    path = os.path.join(HERE, "adjoint_fd_cyl400.json")
    with open(path, "w") as fp:
        json.dump(out, fp, indent=1)
    print(path, json.dumps(out)[:400])


if __name__ == "__main__":
    main()
