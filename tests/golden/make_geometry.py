"""The reference's geometry reader on prefab bodies, as marker data.

Runs the reference's serial build of ``oracle/cases/fem_filament_d2q9.h``
(IBM and the geometry reader on) for 0 steps with a geometry.config holding
an IB circle (CIRCLE_SPHERE IBM ... RIGID) and a FILAMENT_ARRAY of two
flexible filaments (CONFORMING elements), and stores the config text and,
per marker, body, index, position, epsilon and ds after ibm_initialise.

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

CASE = "fem_filament_d2q9"
CONFIG = ("# a rigid IB circle and two flexible filaments\n"
          "CIRCLE_SPHERE IBM 0 0 1.2 0.5 0.0 0.15 RIGID\n"
          "FILAMENT_ARRAY IBM 0 0 2 0.4 0.0 0.0 0.3 0.0 0.0 0.3 0.02 0.0 90.0 0.0 FLEXIBLE CONFORMING CLAMPED "
          "1000.0 100000000.0\n")


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    a = ap.parse_args()
    exe = build_ref.build_case(CASE, a.ref)
    work = tempfile.mkdtemp(prefix="geom_")
    os.makedirs(os.path.join(work, "input"))
    with open(os.path.join(work, "input", "geometry.config"), "w") as fp:
        fp.write(CONFIG)
    subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0",
                    "--workdir", work], check=True)
    mk = np.loadtxt(os.path.join(work, "out", "s0", "markers.txt"), ndmin=2)
    # columns: body, marker, x, y, z, Fx, Fy, Fz, epsilon, ds, ...
    rows = [[int(r[0]), int(r[1]), *map(float, r[2:5]), float(r[8]), float(r[9])] for r in mk]
    dst = os.path.join(HERE, "geometry_prefab.json")
    with open(dst, "w") as fp:
        json.dump({"case": CASE, "config": CONFIG, "markers": rows}, fp, indent=0)
    print(dst, len(rows))
    return 0


if __name__ == "__main__":
    sys.exit(main())
