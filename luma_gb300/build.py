"""Build the in-tree CUDA library ``luma_gb300/_build/libluma_gpu.so``.

Compiles every ``csrc/*.cu`` translation unit for sm_103a in parallel with
nvcc and links them into one shared library exporting the C ABI declared in
``include/luma_gpu.h``.  Incremental: a unit is recompiled when it or any
header under ``csrc/`` or ``include/`` is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libluma_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Units whose FP64 operation sequence must be the reference's (no FMA contraction).
FMAD_OFF = {"fem.cu", "epsilon.cu"}
# Units compiled once per variant (object suffix, defines): the general-path
# kernels instantiate per lattice and precision, six objects in parallel.
VARIANTS = {
    "k_general.cu": [(f"q{q}_{p}", [f"-DLUMA_GEN_Q={q}", f"-DLUMA_GEN_FP64={1 if p == 'fp64' else 0}"])
                     for q in (9, 19, 27) for p in ("fp64", "fp32")],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build luma_gb300")


def _flags(debug: bool) -> list[str]:
    f = ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]
    if debug:
        f += ["-DLUMA_GPU_CHECKS=1"]
    return f


def build(force: bool = False, debug: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))
    newest_hdr = max((os.path.getmtime(h) for h in headers), default=0)
    cc = nvcc()
    flags = _flags(debug)

    jobs_list = []
    for src in units:
        base = os.path.basename(src)
        for suffix, defs in VARIANTS.get(base, [("", [])]):
            obj = os.path.join(BUILD, base[:-3] + (f"_{suffix}" if suffix else "") + ".o")
            jobs_list.append((src, obj, defs))

    def compile_one(job):
        src, obj, defs = job
        if not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), newest_hdr):
            return obj, None
        extra = ["-fmad=false"] if os.path.basename(src) in FMAD_OFF else []
        cmd = [cc, *flags, *extra, *defs, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return obj, " ".join(cmd) + "\n" + r.stdout[-3000:] + r.stderr[-6000:]
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj, None

    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_list), os.cpu_count() or 4)) as ex:
        res = list(ex.map(compile_one, jobs_list))
    errs = [e for _, e in res if e]
    if errs:
        raise RuntimeError("luma_gb300 CUDA build failed:\n" + "\n".join(errs))
    objs = [o for o, _ in res]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("luma_gb300 link failed:\n" + r.stderr[-4000:])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
