"""The reference's own ASCII writers on an oracle case, as SHA-256 digests.

Builds ``oracle/cases/refine_d2q9.h`` (D2Q9 channel with one refined
region), ``tavg_refine_d2q9.h`` (the same with time-averaged quantities,
whose io_lite lines carry them) and ``ibm_cyl_d2q9.h`` (an IB cylinder:
the restart also writes the bodies' marker file) with the reference's serial
build, runs 12 steps and calls
GridObj::io_lite(12, "") and GridObj::io_restart(eWrite) after the last
(harness option ``--io-at``).  Stores, per written file, its size and the
SHA-256 of its bytes (the files themselves are 1.8 MB of text).  Then runs
the reference's reader, GridObj::io_restart(eRead), on that restart file
(``--restart-read``) and stores the SHA-256 of every grid's f, u and rho as
it leaves them.

Output: ``io_<case>.json`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_io.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py)
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402
from tests.golden import cases as CASE_DEFS  # noqa: E402

CASES, STEPS, PRECISION = ("refine_d2q9", "tavg_refine_d2q9", "ibm_cyl_d2q9"), 12, 10  # L_OUTPUT_PRECISION


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    a = ap.parse_args()
    for case in CASES:
        exe = build_ref.build_case(case, a.ref)
        work = tempfile.mkdtemp(prefix="io_")
        extra = []
        if CASE_DEFS.bodies(case):
            mpath = os.path.join(work, "markers.in")
            CASE_DEFS.write_marker_file(mpath, CASE_DEFS.bodies(case))
            extra = ["--markers", mpath]
        subprocess.run([exe, "--out", work, "--steps", str(STEPS), "--dump-every", "0", "--io-at", str(STEPS),
                        *extra], check=True)
        files = {}
        for name in sorted(os.listdir(work)):
            if name.startswith(("io_lite.", "restart_LBM_", "restart_IBBody_")):
                data = open(os.path.join(work, name), "rb").read()
                files[name] = {"bytes": len(data), "sha256": hashlib.sha256(data).hexdigest()}
        back = tempfile.mkdtemp(prefix="io_read_")
        os.makedirs(os.path.join(back, "input"))
        for name in ("restart_LBM_Rnk0.out", "restart_IBBody_Rnk0.out"):
            if os.path.exists(os.path.join(work, name)):
                shutil.copy(os.path.join(work, name), os.path.join(back, "input"))
        subprocess.run([exe, "--out", os.path.join(back, "out"), "--steps", "0", "--dump-every", "0",
                        "--workdir", back, "--restart-read", *extra], check=True)
        read = {}
        s0 = os.path.join(back, "out", "s0")
        for name in sorted(os.listdir(s0)):
            if name.endswith(("_f.bin", "_u.bin", "_rho.bin")):
                data = np.fromfile(os.path.join(s0, name), dtype=np.float64)
                read[name[:-4]] = hashlib.sha256(data.tobytes()).hexdigest()
        out = {"case": case, "steps": STEPS, "precision": PRECISION, "files": files, "restart_read": read}
        dst = os.path.join(HERE, f"io_{case}.json")
        with open(dst, "w") as fp:
            json.dump(out, fp, indent=1)
        print(dst)
    return 0


if __name__ == "__main__":
    sys.exit(main())
