"""The reference's momentum-exchange force for the momex case.

Builds ``oracle/cases/momex_d2q9.h`` (the Poiseuille channel of the
``poiseuille_d2q9`` case compiled with L_LD_OUT) from the reference checkout
and runs it with ``--momex-out``: per step s, the force
ObjectManager::computeLiftDrag (src/ObjectManager.cpp:93-165) accumulates
over the solid sites during step s, from the populations before it.

Output: ``momex_d2q9.json`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_momex.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py) [--steps 300]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    ap.add_argument("--steps", type=int, default=300)
    a = ap.parse_args()
    exe = build_ref.build_case("momex_d2q9", a.ref)
    work = tempfile.mkdtemp(prefix="momex_")
    path = os.path.join(work, "momex.txt")
    subprocess.run([exe, "--out", work, "--steps", str(a.steps), "--dump-every", "0", "--momex-out", path],
                   check=True, capture_output=True)
    forces = {}
    with open(path) as fp:
        for line in fp:
            s, fx, fy, fz = line.split()
            forces[int(s)] = [float(fx), float(fy), float(fz)]
    out = {"case": "momex_d2q9", "like": "poiseuille_d2q9", "steps": a.steps,
           "note": "forces[s] = accumulated during step s from the populations after step s-1",
           "forces": {str(s): forces[s] for s in sorted(forces)}}
    dst = os.path.join(HERE, "momex_d2q9.json")
    with open(dst, "w") as fp:
        json.dump(out, fp)
    print(dst, forces[1], forces[a.steps])


if __name__ == "__main__":
    main()
