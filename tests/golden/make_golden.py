"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own serial build (``oracle/build_ref.py`` compiles it
from the reference checkout into ``oracle/_ref/<case>/luma_ref``) on each
oracle case, with seeded injected initial fields where the case needs them,
and stores the inputs the reference computed plus its outputs at chosen
steps.  Large population arrays are stored as SHA-256 digests of their raw
FP64 bytes (bit-exact checks need no copy of the data).

Also extracts the one known-answer vector the reference's own test suite
holds for the current algorithm: the t=0 D2Q9 equilibrium row of
``cases/testsuite/base/case000/io_lite.Lev0.Reg0.Rnk0.0.dat``.

Usage (needs the reference checkout; not run on the GPU machine):
    python tests/golden/make_golden.py [--ref LUMA_DIR]  (default: $LUMA_REFERENCE_DIR, see oracle/build_ref.py) [case ...]
"""
from __future__ import annotations

import argparse
import hashlib
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
from tests.golden import cases as CASES  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def read_grid(d: str, lev: int = 0, reg: int = 0) -> dict:
    p = os.path.join(d, f"L{lev}R{reg}_")
    meta = {}
    with open(p + "meta.txt") as fp:
        for line in fp:
            k, *v = line.split()
            meta[k] = [float(x) if "." in x or "e" in x else int(x) for x in v]
            if len(meta[k]) == 1:
                meta[k] = meta[k][0]
    out = {"meta": meta}
    for name in ("f", "u", "rho", "uxin", "xpos", "ypos", "zpos", "force", "rho_ta", "ui_ta", "uiuj_ta"):
        if os.path.exists(p + name + ".bin"):
            out[name] = np.fromfile(p + name + ".bin", dtype=np.float64)
    out["typ"] = np.fromfile(p + "typ.bin", dtype=np.int32)
    return out


def run_case(name: str, ref: str) -> str:
    spec = CASES.CASES[name]
    exe = build_ref.build_case(name, ref)
    work = tempfile.mkdtemp(prefix=f"golden_{name}_")
    args = [exe, "--out", work, "--steps", str(max(spec["steps"])), "--dump-every", "0"]
    init = CASES.initial_fields(name)
    if init is not None:
        upath = os.path.join(work, "init_u.bin")
        init["u"].astype(np.float64).tofile(upath)
        args += ["--init-u", upath]
    if spec.get("filaments") or spec.get("bfl"):
        os.makedirs(os.path.join(work, "input"), exist_ok=True)
        with open(os.path.join(work, "input", "geometry.config"), "w") as fp:
            fp.write(CASES.geometry_config(name))
        args += ["--workdir", work]
    if spec.get("bfl"):
        args += ["--bfl-out", os.path.join(work, "bfl.txt"), "--bfl-forces", os.path.join(work, "bfl_forces.txt")]
    blist = CASES.bodies(name) or (["filament"] if spec.get("filaments") else [])
    if blist and not spec.get("filaments"):
        mpath = os.path.join(work, "markers.in")
        CASES.write_marker_file(mpath, blist)
        args += ["--markers", mpath]
    # Dump at each requested step: rerun with --dump-every = gcd is wasteful;
    # the harness dumps every `dump-every` steps, so pick the gcd of steps.
    g = 0
    for s in spec["steps"]:
        g = np.gcd(g, s)
    args[args.index("--dump-every") + 1] = str(int(g))
    subprocess.run(args, check=True)
    out = {"case": name}
    levels = [(0, 0)] + [(l + 1, 0) for l in range(len(spec.get("regions", [])))]
    s0 = read_grid(os.path.join(work, "s0"))
    out["omega"] = np.float64(s0["meta"]["omega"])
    out["typ"] = s0["typ"]
    out["ux_in"] = s0["uxin"]
    out["ypos"] = s0["ypos"]
    out["f0_sha"] = sha(s0["f"])
    for (lev, reg) in levels[1:]:
        gl = read_grid(os.path.join(work, "s0"), lev, reg)
        k = f"L{lev}R{reg}"
        out[f"{k}_typ"] = gl["typ"]
        out[f"{k}_omega"] = np.float64(gl["meta"]["omega"])
        out[f"{k}_coarse_lims"] = np.array(gl["meta"]["coarse_lims"], dtype=np.int64)
        out[f"{k}_xpos"] = gl["xpos"]
        out[f"{k}_ypos"] = gl["ypos"]
        out[f"{k}_zpos"] = gl["zpos"]
        out[f"{k}_ux_in"] = gl["uxin"]
        out[f"{k}_f0_sha"] = sha(gl["f"])
    if init is not None and spec.get("store_fields", True):
        out["init_u"] = init["u"]
    for s in spec["steps"]:
        gs = read_grid(os.path.join(work, f"s{s}"))
        if spec.get("store_fields", True):
            out[f"u_{s}"] = gs["u"]
            out[f"rho_{s}"] = gs["rho"]
        if spec.get("store_tav"):
            for t in ("rho_ta", "ui_ta", "uiuj_ta"):
                out[f"{t}_{s}"] = gs[t]
                for (lev, reg) in levels[1:]:
                    out[f"L{lev}R{reg}_{t}_{s}"] = read_grid(os.path.join(work, f"s{s}"), lev, reg)[t]
        out[f"u_sha_{s}"] = sha(gs["u"])
        out[f"rho_sha_{s}"] = sha(gs["rho"])
        out[f"f_sha_{s}"] = sha(gs["f"])
        if s in spec.get("store_f", ()):
            out[f"f_{s}"] = gs["f"]
        for (lev, reg) in levels[1:]:
            gl = read_grid(os.path.join(work, f"s{s}"), lev, reg)
            k = f"L{lev}R{reg}"
            if spec.get("store_fields", True):
                out[f"{k}_u_{s}"] = gl["u"]
                out[f"{k}_rho_{s}"] = gl["rho"]
            out[f"{k}_u_sha_{s}"] = sha(gl["u"])
            out[f"{k}_rho_sha_{s}"] = sha(gl["rho"])
            out[f"{k}_f_sha_{s}"] = sha(gl["f"])
    if blist:
        for s in (0,) + tuple(spec["steps"]):
            mk = np.loadtxt(os.path.join(work, f"s{s}", "markers.txt"), ndmin=2)
            out[f"markers_{s}"] = mk
        sup = np.loadtxt(os.path.join(work, "s0", "supports.txt"), ndmin=2)
        out["supports"] = sup
    if spec.get("bfl"):
        with open(os.path.join(work, "bfl.txt")) as fp:
            lines = fp.read().split("\n")
        nm, q = (int(x) for x in lines[0].split())
        out["bfl_q"] = np.array([[float(x) for x in lines[1 + m].split()] for m in range(nm)]).reshape(nm, q)
        out["bfl_site_marker"] = np.array([int(x) for x in lines[1 + nm:] if x.strip()], dtype=np.int32)
        bf = np.loadtxt(os.path.join(work, "bfl_forces.txt"), ndmin=2)
        forces = bf[:, 2:5].reshape(-1, nm, 3)
        keep = sorted(set(range(1, min(10, len(forces)) + 1)) | set(spec["steps"]))
        out["bfl_force_steps"] = np.array(keep, dtype=np.int64)
        out["bfl_forces"] = forces[np.array(keep) - 1]
    with open(os.path.join(work, "timing.txt")) as fp:
        out["ref_timing"] = fp.read()
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return work


def extract_kat(ref: str) -> None:
    path = os.path.join(ref, "cases", "testsuite", "base", "case000", "io_lite.Lev0.Reg0.Rnk0.0.dat")
    with open(path) as fp:
        lines = fp.read().splitlines()
    head = lines[2].split()
    row = lines[3].split()
    col = {h: i for i, h in enumerate(head)}
    rec = {
        "source": "LUMA cases/testsuite/base/case000/io_lite.Lev0.Reg0.Rnk0.0.dat, first data row",
        "rho": float(row[col["RHO"]]),
        "u": [float(row[col["UX"]]), float(row[col["UY"]])],
        "f": [float(row[col[f"F{v}"]]) for v in range(9)],
        "decimals": 8,
    }
    with open(os.path.join(HERE, "kat_feq_d2q9.json"), "w") as fp:
        json.dump(rec, fp, indent=1)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=build_ref.DEFAULT_REF)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args(argv)
    extract_kat(a.ref)
    for c in a.cases or sorted(CASES.CASES):
        print(c, run_case(c, a.ref))
    return 0


if __name__ == "__main__":
    sys.exit(main())
