"""The reference's geometry reader on prefab bodies, as marker data.

Runs the reference's serial build for 0 steps with a geometry.config and
stores the config text and, per marker, body, index, position, epsilon and
ds after ibm_initialise:
* ``oracle/cases/fem_filament_d2q9.h`` (2D, IBM and the reader on): an IB
  circle, a FILAMENT_ARRAY of two flexible filaments (CONFORMING elements),
  a rotated square and a rigid filament;
* ``oracle/cases/geom_d3q19.h`` (3D): a sphere, a rotated cube, a plate and
  two rigid filaments.

Output: ``geometry_prefab.json`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_geometry.py [--ref /root/reference/LUMA]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402

RUNS = {
    "fem_filament_d2q9": ("# a rigid IB circle, two flexible filaments, a square and a rigid filament\n"
                          "CIRCLE_SPHERE IBM 0 0 1.2 0.5 0.0 0.15 RIGID\n"
                          "FILAMENT_ARRAY IBM 0 0 2 0.4 0.0 0.0 0.3 0.0 0.0 0.3 0.02 0.0 90.0 0.0 FLEXIBLE "
                          "CONFORMING CLAMPED 1000.0 100000000.0\n"
                          "SQUARE_CUBE IBM 0 0 1.6 0.45 0.0 0.2 0.1 0.0 30.0 0.0 RIGID\n"
                          "FILAMENT_ARRAY IBM 0 0 1 1.85 0.1 0.0 0.0 0.0 0.0 0.3 0.02 0.0 80.0 0.0 RIGID "
                          "CONFORMING CLAMPED 1000.0 100000000.0\n"),
    "geom_d3q19": ("CIRCLE_SPHERE IBM 0 0 0.4 0.45 0.5 0.15 RIGID\n"
                   "SQUARE_CUBE IBM 0 0 0.9 0.45 0.5 0.3 0.2 0.2 20.0 10.0 RIGID\n"
                   "PLATE IBM 0 0 1.4 0.5 0.5 0.3 0.2 10.0 20.0 30.0 RIGID\n"
                   "FILAMENT_ARRAY IBM 0 0 2 1.75 0.0 0.3 0.0 0.0 0.3 0.4 0.05 0.05 70.0 25.0 MOVABLE "
                   "CONFORMING CLAMPED 1000.0 100000000.0\n"),
}


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    a = ap.parse_args()
    runs = []
    for case, config in RUNS.items():
        exe = build_ref.build_case(case, a.ref)
        work = tempfile.mkdtemp(prefix="geom_")
        os.makedirs(os.path.join(work, "input"))
        with open(os.path.join(work, "input", "geometry.config"), "w") as fp:
            fp.write(config)
        subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0",
                        "--workdir", work], check=True)
        mk = np.loadtxt(os.path.join(work, "out", "s0", "markers.txt"), ndmin=2)
        # columns: body, marker, x, y, z, Fx, Fy, Fz, epsilon, ds, ...
        rows = [[int(r[0]), int(r[1]), *map(float, r[2:5]), float(r[8]), float(r[9])] for r in mk]
        runs.append({"case": case, "config": config, "markers": rows})
        print(case, len(rows))
    dst = os.path.join(HERE, "geometry_prefab.json")
    with open(dst, "w") as fp:
        json.dump({"runs": runs}, fp, indent=0)
    print(dst)
    return 0


if __name__ == "__main__":
    sys.exit(main())
