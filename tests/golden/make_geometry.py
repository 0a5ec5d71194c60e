"""The reference's geometry reader on prefab bodies, as marker data.

Runs the reference's serial build for 0 steps with a geometry.config and
stores the config text and, per marker, body, index, position, epsilon and
ds after ibm_initialise:
* ``oracle/cases/fem_filament_d2q9.h`` (2D, IBM and the reader on): an IB
  circle, a FILAMENT_ARRAY of two flexible filaments (CONFORMING elements),
  a rotated square and a rigid filament;
* ``oracle/cases/geom_d3q19.h`` (3D): a sphere, a rotated cube, a plate and
  two rigid filaments;
* ``oracle/cases/ibm_universal_d2q9.h`` (2D, L_UNIVERSAL_EPSILON_CALC): two
  circles whose supports overlap and a square;
* ``oracle/cases/geom_refine_d2q9.h`` (2D, one refined region) for the
  point clouds placed on level 1.

Output: ``geometry_prefab.json`` beside this script.

FROM_FILE point clouds (seeded synthetic clouds written here): for each run
of ``CLOUD_RUNS`` the cloud files go to the run's ``input/`` folder and
``geometry_cloud.npz`` stores the cloud texts, the config, the level-0
labels, velocity and density of every grid after the reader (BBB
labelling; one run puts clouds on a refined level), the IB
markers (as above) and, for BFL runs, the body's Q table and per-site marker
lookup (``--bfl-out``).

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_geometry.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py)
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
    "ibm_universal_d2q9": ("# two circles whose supports overlap and a square, one epsilon system\n"
                           "CIRCLE_SPHERE IBM 0 0 0.9 0.5 0.0 0.1 RIGID\n"
                           "CIRCLE_SPHERE IBM 0 0 1.135 0.5 0.0 0.1 RIGID\n"
                           "SQUARE_CUBE IBM 0 0 1.6 0.45 0.0 0.15 0.1 0.0 20.0 0.0 RIGID\n"),
}


def _cloud_texts() -> dict:
    """Seeded clouds: a 2D cambered ellipse (700 points, final newline: the
    reader repeats the last point), a filled 2D disc, a 2D bar, a 3D
    ellipsoid surface (1500 points) and a filled 3D box with one line of
    two values (the reader keeps the previous z)."""
    rs = np.random.RandomState(7)
    t = np.linspace(0.0, 2.0 * np.pi, 700, endpoint=False)
    ell = np.stack([np.cos(t), 0.35 * np.sin(t) + 0.05 * np.sin(2 * t)], 1) + rs.uniform(-1e-3, 1e-3, (700, 2))
    xs, ys = np.meshgrid(np.linspace(-1, 1, 41), np.linspace(-1, 1, 41))
    keep = xs ** 2 + ys ** 2 <= 1.0
    disc = np.stack([xs[keep], ys[keep]], 1)
    bar = np.stack([np.linspace(0.0, 5.0, 200), 0.02 * np.sin(np.linspace(0.0, 9.0, 200))], 1)
    n = 1500
    k = np.arange(n) + 0.5
    phi = np.arccos(1.0 - 2.0 * k / n)
    th = np.pi * (1.0 + 5.0 ** 0.5) * k
    sph = np.stack([2.0 * np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), 0.8 * np.cos(phi)], 1)
    sph += rs.uniform(-1e-3, 1e-3, sph.shape)
    g = np.linspace(0.0, 1.0, 9)
    box = np.stack(np.meshgrid(g, 0.5 * g, 0.7 * g, indexing="ij"), -1).reshape(-1, 3)
    lines = ["%.6f %.6f %.6f" % tuple(p) for p in box]
    lines[300] = "%.6f %.6f" % tuple(box[300, :2])
    return {
        "ellipse.txt": "".join("%.6f %.6f\n" % tuple(p) for p in ell),
        "disc.txt": "\n".join("%.6f %.6f" % tuple(p) for p in disc),
        "bar.txt": "\n".join("%.6f %.6f" % tuple(p) for p in bar) + "\n",
        "ellipsoid.txt": "\n".join("%.6f %.6f %.6f" % tuple(p) for p in sph),
        "box.txt": "\n".join(lines) + "\n",
    }


CLOUD_RUNS = {
    "ibm_bbb_2d": ("fem_filament_d2q9",
                   "FROM_FILE IBM ellipse.txt 0 0 CENTRE 0.6 CENTRE 0.5 START 0.0 0.4 X RIGID CLAMPED\n"
                   "FROM_FILE BBB disc.txt 0 0 START 1.3 CENTRE 0.5 START 0.0 0.2 Y RIGID CLAMPED\n"
                   "FROM_FILE BBB bar.txt 0 0 START 1.7 START 0.9 START 0.0 0.5 X RIGID CLAMPED\n"),
    "bfl_2d": ("bfl_cyl_d2q9",
               "FROM_FILE BFL ellipse.txt 0 0 CENTRE 0.7 CENTRE 0.5 START 0.0 0.3 X RIGID CLAMPED\n"),
    "ibm_bbb_3d": ("geom_d3q19",
                   "FROM_FILE IBM ellipsoid.txt 0 0 CENTRE 0.5 CENTRE 0.5 CENTRE 0.5 0.4 X RIGID CLAMPED\n"
                   "FROM_FILE BBB box.txt 0 0 START 1.2 START 0.1 CENTRE 0.5 0.2 Z RIGID CLAMPED\n"),
    "bfl_3d": ("bfl_sphere_d3q19",
               "FROM_FILE BFL ellipsoid.txt 0 0 CENTRE 0.6 CENTRE 0.5 CENTRE 0.5 0.4 X RIGID CLAMPED\n"),
    "levels_2d": ("geom_refine_d2q9",
                  "FROM_FILE IBM ellipse.txt 1 0 CENTRE 0.7 CENTRE 0.55 START 0.0 0.15 X RIGID CLAMPED\n"
                  "FROM_FILE BBB disc.txt 1 0 CENTRE 0.9 CENTRE 0.4 START 0.0 0.08 X RIGID CLAMPED\n"
                      "FROM_FILE BBB bar.txt 1 0 START 0.6 START 0.3 START 0.0 0.5 X RIGID CLAMPED\n"
                      "FROM_FILE BBB disc.txt 0 0 START 1.4 CENTRE 0.5 START 0.0 0.15 Y RIGID CLAMPED\n"),
}


def _level0(path: str):
    out = {}
    for k, dt in (("typ", np.int32), ("u", np.float64), ("rho", np.float64)):
        out[k] = np.fromfile(path + k + ".bin", dtype=dt)
    return out


def make_clouds(ref: str) -> str:
    clouds = _cloud_texts()
    store = {}
    for run, (case, config) in CLOUD_RUNS.items():
        exe = build_ref.build_case(case, ref)
        work = tempfile.mkdtemp(prefix="cloud_")
        os.makedirs(os.path.join(work, "input"))
        with open(os.path.join(work, "input", "geometry.config"), "w") as fp:
            fp.write(config)
        for fname, text in clouds.items():
            with open(os.path.join(work, "input", fname), "w") as fp:
                fp.write(text)
        bfl = os.path.join(work, "bfl.txt")
        subprocess.run([exe, "--out", os.path.join(work, "out"), "--steps", "0", "--dump-every", "0",
                        "--workdir", work, "--bfl-out", bfl], check=True, timeout=600)
        store[run + "/case"] = np.array(case)
        store[run + "/config"] = np.array(config)
        for meta in sorted(os.listdir(os.path.join(work, "out", "s0"))):
            if meta.endswith("_meta.txt"):
                key = meta[:-len("_meta.txt")]
                for k, v in _level0(os.path.join(work, "out", "s0", key + "_")).items():
                    store[run + "/" + key + "/" + k] = v
        mk_path = os.path.join(work, "out", "s0", "markers.txt")
        if os.path.exists(mk_path):
            mk = np.loadtxt(mk_path, ndmin=2)
            store[run + "/markers"] = np.array([[r[0], r[1], *r[2:5], r[8], r[9]] for r in mk], dtype=np.float64)
        lines = open(bfl).read().split("\n")
        nm, q = (int(x) for x in lines[0].split())
        if nm:
            store[run + "/bfl_q"] = np.array([[float(x) for x in lines[1 + m].split()] for m in range(nm)])
            store[run + "/bfl_marker"] = np.array([int(x) for x in lines[1 + nm:] if x.strip()], dtype=np.int32)
        print(run, case, "markers" if os.path.exists(mk_path) else "", nm)
    for fname, text in clouds.items():
        store["cloud/" + fname] = np.array(text)
    dst = os.path.join(HERE, "geometry_cloud.npz")
    np.savez_compressed(dst, **store)
    return dst


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    ap.add_argument("--clouds-only", action="store_true")
    a = ap.parse_args()
    if a.clouds_only:
        print(make_clouds(a.ref))
        return 0
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
    print(make_clouds(a.ref))
    return 0


if __name__ == "__main__":
    sys.exit(main())
