"""Oracle test infrastructure: build the reference's own serial LUMA code.

Compiles the reference translation units where they lie (``LUMA/src`` under
the reference checkout, never copied) once per oracle case, with that case's
configuration header pre-included in place of the reference's
``inc/definitions.h`` (same include guard), the type-only ``mpi.h`` shim, the
stubs in ``ref_stubs.cpp`` and the driver ``ref_harness.cpp``.  Outputs go to
``oracle/_ref/<case>/`` only.

Left out of the build: ``main_lbm.cpp`` (the harness replaces it) and the
``MpiManager*.cpp`` / ``Mpi_buffer_*.cpp`` sources (MPI calls outside
``L_BUILD_FOR_MPI`` guards).  ``GridObj_ops_io.cpp`` includes ``hdf5.h``
unconditionally; it compiles against the do-nothing ``shim/hdf5.h`` (its
HDF5 writer is never called) for its ASCII writers.

Usage: ``python oracle/build_ref.py [--ref LUMA_DIR] [case ...]`` (default
``$LUMA_REFERENCE_DIR``).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CASES_DIR = os.path.join(HERE, "cases")
OUT_ROOT = os.path.join(HERE, "_ref")
# The reference checkout's LUMA directory: $LUMA_REFERENCE_DIR, else the place
# this recipe's build container holds it.  Only this recipe and the fixture
# scripts under tests/golden/ read the reference; nothing at run time does.
REF_ENV = "LUMA_REFERENCE_DIR"
DEFAULT_REF = os.environ.get(REF_ENV) or "/root/reference/LUMA"

EXCLUDE_PREFIX = ("main_lbm", "MpiManager", "Mpi_buffer")


def list_cases() -> list[str]:
    return sorted(f[:-2] for f in os.listdir(CASES_DIR)
                  if f.endswith(".h") and not f.startswith("luma_case_tail"))


def _compile(args):
    src, obj, flags = args
    if os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src):
        return None
    cmd = ["gcc" if src.endswith(".c") else "g++", *flags, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return f"{' '.join(cmd)}\n{r.stderr[-4000:]}"
    return None


ROOT = os.path.dirname(HERE)
SHIM_DIR = os.path.join(ROOT, "luma_gb300", "shim")
GPU_LIB_DIR = os.path.join(ROOT, "luma_gb300", "_build")
SHIM_BACKENDS = ("oracle", "gpu")


def build_case(case: str, ref: str = DEFAULT_REF, jobs: int | None = None, shim: str | None = None) -> str:
    """Build ``oracle/_ref/<case>/luma_ref``; return the binary path.

    With ``shim`` the harness is built with the LUMA-side shim
    (``luma_gb300/shim/gridobj_gpu.cpp``, compiled against the reference's
    own headers) into ``oracle/_ref/<case>_shim_<shim>/``: ``"gpu"`` links
    ``libluma_gpu.so`` (the drop-in as a maintainer builds it), ``"oracle"``
    links the shim's ABI calls to the oracle (``abi_on_oracle.c``) so the
    shim runs on the host."""
    src_dir = os.path.join(ref, "src")
    out = os.path.join(OUT_ROOT, case if shim is None else f"{case}_shim_{shim}")
    os.makedirs(out, exist_ok=True)
    header = os.path.join(CASES_DIR, case + ".h")
    flags = ["-O2", "-std=c++11", "-w", "-ffp-contract=off",
             "-I", os.path.join(HERE, "shim"), "-I", CASES_DIR, "-I", src_dir,
             "-include", header, "-include", os.path.join(HERE, "ref_prefix.h")]
    if shim is not None:
        if shim not in SHIM_BACKENDS:
            raise ValueError(f"shim backend {shim!r} not in {SHIM_BACKENDS}")
        flags = flags + ["-DLUMA_HARNESS_SHIM", "-I", SHIM_DIR, "-I", os.path.join(ref, "inc")]
    units = []
    for f in sorted(os.listdir(src_dir)):
        if not f.endswith(".cpp") or f.startswith(EXCLUDE_PREFIX):
            continue
        units.append((os.path.join(src_dir, f), os.path.join(out, f[:-4] + ".o"), flags))
    for f in ("ref_stubs.cpp", "ref_harness.cpp"):
        units.append((os.path.join(HERE, f), os.path.join(out, f[:-4] + ".o"), flags))
    extra_deps = []
    if shim is not None:
        units.append((os.path.join(SHIM_DIR, "gridobj_gpu.cpp"), os.path.join(out, "gridobj_gpu.o"), flags))
        extra_deps = [os.path.join(SHIM_DIR, "gridobj_gpu.cpp"), os.path.join(SHIM_DIR, "gridobj_gpu.h"),
                      os.path.join(ROOT, "include", "luma_gpu.h")]
        if shim == "oracle":
            cflags = ["-O2", "-std=c11", "-w", "-ffp-contract=off", "-fopenmp"]
            for f in ("abi_on_oracle.c", "lbm_oracle.c"):
                units.append((os.path.join(HERE, f), os.path.join(out, f[:-2] + ".o"), cflags))
                extra_deps.append(os.path.join(HERE, f))
    # A changed case header or harness invalidates every object of the case.
    stamp = os.path.join(out, ".stamp")
    deps = [header, os.path.join(CASES_DIR, "luma_case_tail.h"), os.path.join(HERE, "ref_prefix.h"),
            os.path.join(HERE, "ref_stubs.cpp"), os.path.join(HERE, "ref_harness.cpp"), *extra_deps]
    newest = max(os.path.getmtime(d) for d in deps)
    if not os.path.exists(stamp) or os.path.getmtime(stamp) < newest:
        for _, obj, _ in units:
            if os.path.exists(obj):
                os.remove(obj)
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        errs = [e for e in ex.map(_compile, units) if e]
    if errs:
        raise RuntimeError("oracle reference build failed:\n" + "\n".join(errs))
    exe = os.path.join(out, "luma_ref")
    libs = []
    if shim == "oracle":
        libs = ["-fopenmp", "-lm"]
    elif shim == "gpu":
        libs = ["-L", GPU_LIB_DIR, "-lluma_gpu", f"-Wl,-rpath,{GPU_LIB_DIR}"]
    r = subprocess.run(["g++", "-o", exe, *[u[1] for u in units], *libs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle reference link failed:\n" + r.stderr[-4000:])
    with open(stamp, "w") as fp:
        fp.write("ok\n")
    return exe


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("cases", nargs="*")
    a = ap.parse_args(argv)
    if not os.path.isdir(a.ref):
        print(f"reference not found at {a.ref}; nothing to build", file=sys.stderr)
        return 0
    for c in a.cases or list_cases():
        print(build_case(c, a.ref))
    return 0


if __name__ == "__main__":
    sys.exit(main())
