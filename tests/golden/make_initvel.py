"""The reference's initial-velocity reader (L_INIT_VELOCITY_FROM_FILE) on
seeded velocity files, as level-0 velocity and populations; and its
inlet-profile reader (L_USE_INLET_PROFILE) on a refined channel.

Builds ``oracle/cases/initvel_d2q9.h`` (2D channel 40 x 20) and
``initvel_d3q19.h`` (periodic 12 x 8 x 6) with the reference's serial
build, writes ``input/initial_velocity.in`` and runs 0 steps; stores the
file text and the level-0 u and f the reference starts from.  The files
list every site once at a jittered position inside it plus duplicates and
points off the grid, shuffled, with a final newline; the 2D file's
ordering leaves some sites unset (only the first N*M*K points count) and
the 3D file has a short line among the last points that count (every later
value repeats the last one read).

``oracle/cases/inletfile_refine_d2q9.h`` (80 x 40 channel with a refined
region) reads ``input/inlet_profile.in`` (five points, a final newline);
stored: the text and every grid's inlet profile, velocity and populations.

``oracle/cases/refine_halfcell_d2q9.h`` (16 x 8 channel whose refined
region's limits fall on half coarse cells): every grid's labels and site
positions, which pin the std::round of the sub-grid edges.

Output: ``initial_velocity.npz`` beside this script.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_initvel.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py)
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build_ref  # noqa: E402

RUNS = {"initvel_d2q9": ((40, 20, 1), 1.0 / 20), "initvel_d3q19": ((12, 8, 6), 1.0 / 4)}


def velocity_text(case: str, seed: int) -> str:
    (N, M, K), dh = RUNS[case]
    rs = np.random.RandomState(seed)
    ii, jj, kk = np.meshgrid(np.arange(N), np.arange(M), np.arange(K), indexing="ij")
    pos = np.stack([ii, jj, kk], -1).reshape(-1, 3) + rs.uniform(0.05, 0.95, (N * M * K, 3))
    pos *= dh
    extra = pos[rs.choice(len(pos), 25)] + rs.uniform(-0.4, 0.4, (25, 3)) * dh
    off = rs.uniform(-0.5, 0.5, (6, 3)) + np.array([N, M, K]) * dh * np.array([1.1, 0.5, 0.5])
    pts = np.concatenate([pos, extra, off])
    if K == 1:
        pts[:, 2] = rs.uniform(-3.0, 3.0, len(pts))  # z is not used in 2D
    vel = rs.uniform(-1.0, 1.0, (len(pts), 3))
    order = rs.permutation(len(pts))
    lines = ["%.9f %.9f %.9f %.9f %.9f %.9f" % (*pts[p], *vel[p]) for p in order]
    if case == "initvel_d3q19":
        cut = N * M * K - 5  # among the points that count
        lines[cut] = " ".join(lines[cut].split()[:4])
    return "\n".join(lines) + "\n"


PROFILE_TEXT = ("0.0 0.1 0.0 0.020 0.001 0.3\n"
                "0.0 0.3 0.0 0.045 -0.002 0.1\n"
                "0.0 0.5125 0.0 0.050 0.000 0.2\n"
                "0.0 0.7 0.0 0.040 0.003 0.4\n"
                "0.0 0.85 0.0 0.025 0.001 0.6\n")


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    a = ap.parse_args()
    store = {}
    for seed, case in enumerate(RUNS):
        exe = build_ref.build_case(case, a.ref)
        work = tempfile.mkdtemp(prefix="initvel_")
        os.makedirs(os.path.join(work, "input"))
        text = velocity_text(case, 11 + seed)
        with open(os.path.join(work, "input", "initial_velocity.in"), "w") as fp:
            fp.write(text)
        subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0",
                        "--workdir", work], check=True, timeout=300)
        s0 = os.path.join(work, "out", "s0", "L0R0_")
        store[case + "/text"] = np.array(text)
        store[case + "/u"] = np.fromfile(s0 + "u.bin", dtype=np.float64)
        store[case + "/f"] = np.fromfile(s0 + "f.bin", dtype=np.float64)
        print(case, len(text.splitlines()), "lines")
    case = "inletfile_refine_d2q9"
    exe = build_ref.build_case(case, a.ref)
    work = tempfile.mkdtemp(prefix="inletfile_")
    os.makedirs(os.path.join(work, "input"))
    with open(os.path.join(work, "input", "inlet_profile.in"), "w") as fp:
        fp.write(PROFILE_TEXT)
    subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0",
                    "--workdir", work], check=True, timeout=300)
    store[case + "/text"] = np.array(PROFILE_TEXT)
    for key in ("L0R0", "L1R0"):
        s0 = os.path.join(work, "out", "s0", key + "_")
        for name in ("uxin", "u", "f"):
            store[f"{case}/{key}/{name}"] = np.fromfile(s0 + name + ".bin", dtype=np.float64)
    print(case)
    case = "refine_halfcell_d2q9"
    exe = build_ref.build_case(case, a.ref)
    work = tempfile.mkdtemp(prefix="halfcell_")
    subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0"], check=True,
                   timeout=300)
    for key in ("L0R0", "L1R0"):
        s0 = os.path.join(work, "out", "s0", key + "_")
        store[f"{case}/{key}/typ"] = np.fromfile(s0 + "typ.bin", dtype=np.int32)
        for name in ("xpos", "ypos"):
            store[f"{case}/{key}/{name}"] = np.fromfile(s0 + name + ".bin", dtype=np.float64)
    print(case)
    dst = os.path.join(HERE, "initial_velocity.npz")
    np.savez_compressed(dst, **store)
    print(dst)
    return 0


if __name__ == "__main__":
    sys.exit(main())
