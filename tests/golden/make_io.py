"""The reference's own ASCII writers on an oracle case, as SHA-256 digests.

Builds ``oracle/cases/refine_d2q9.h`` (D2Q9 channel with one refined
region) and ``tavg_refine_d2q9.h`` (the same with time-averaged
quantities, whose io_lite lines carry them) with the reference's serial
build, runs 12 steps and calls
GridObj::io_lite(12, "") and GridObj::io_restart(eWrite) after the last
(harness option ``--io-at``).  Stores, per written file, its size and the
SHA-256 of its bytes (the files themselves are 1.8 MB of text).

Output: ``io_<case>.json`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_io.py [--ref /root/reference/LUMA]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402

CASES, STEPS, PRECISION = ("refine_d2q9", "tavg_refine_d2q9"), 12, 10   # L_OUTPUT_PRECISION of the cases


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    a = ap.parse_args()
    for case in CASES:
        exe = build_ref.build_case(case, a.ref)
        work = tempfile.mkdtemp(prefix="io_")
        subprocess.run([exe, "--out", work, "--steps", str(STEPS), "--dump-every", "0", "--io-at", str(STEPS)],
                       check=True)
        files = {}
        for name in sorted(os.listdir(work)):
            if name.startswith(("io_lite.", "restart_LBM_")):
                data = open(os.path.join(work, name), "rb").read()
                files[name] = {"bytes": len(data), "sha256": hashlib.sha256(data).hexdigest()}
        out = {"case": case, "steps": STEPS, "precision": PRECISION, "files": files}
        dst = os.path.join(HERE, f"io_{case}.json")
        with open(dst, "w") as fp:
            json.dump(out, fp, indent=1)
        print(dst)
    return 0


if __name__ == "__main__":
    sys.exit(main())
