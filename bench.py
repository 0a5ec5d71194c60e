"""Benchmark: D3Q19 LBGK periodic box 256^3 (tau = 0.55, Taylor-Green
u0 = 0.02 plus seeded 1e-4 noise), million lattice updates per second.

One bench step is one LBM time step of the whole 256^3 grid (GridObj::
LBM_multi_opt on an all-fluid periodic grid).  ``value`` is the shifted-FP32
path (the chosen precision) with the state resident in HBM; the plain FP64
path (the reference's arithmetic) is measured on the same workload and
reported beside it with the FP32-vs-FP64 velocity error.  ``e2e`` goes
through the C ABI with host buffers: upload of the reference-layout FP64
state, the K steps, and download of u and rho, all inside the timed region.

Multi-GPU: every rank runs an independent replica of the box (the path has no
data exchange on one grid per GPU); value = sum over ranks.

The FP32-vs-FP64 accuracy leg runs both paths to t = 10^4 (the stated
accuracy target's step count) whatever ``--steps`` is, outside the timed
regions.

``--impl reference`` times the reference's CPU implementation of the path
(the oracle restatement of GridObj::LBM_multi_opt, bit-exact with the
reference's own serial build, OpenMP over all host threads) on the same
256^3 box, one full-box LBM step per bench step, plus a 1-thread figure.
The same CPU leg gives the ``cpu_baseline`` of the GPU line and, from its
state, the FP64 GPU path's parity at full size.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "D3Q19 MLUPS & %HBM roofline, FP32-shifted vs FP64 at stated error; adjoint cost"
SIZE = 256
TAU = 0.55
# FP64 operations per lattice update of the D3Q19 in-place FP64 kernel
# (dadd + dmul + 2 dfma SASS thread-instruction counters of one launch at
# 128^3, divided by the sites); the FP64 path is bound by the FP64 pipe.
FP64_FLOP_PER_LU_D3Q19 = 231
FP64_NOMINAL_TFLOPS = 1.25
U0 = 0.02
NOISE = 1e-4
ACCURACY_STEPS = 10000      # step count of the FP32-vs-FP64 accuracy target
# a CPU sample (warm-up + timed steps) is kept under this many seconds
CPU_SAMPLE_BUDGET_S = 150.0


def workload_level0(n: int, nz: int | None = None):
    """Level-0 grid of the periodic Taylor-Green box (n x n x nz)."""
    from luma_gb300 import _abi as A
    from luma_gb300 import case as hostcase
    from tests.golden.cases import taylor_green
    nz = nz or n
    # dt = dh/16 keeps the reference's Mach check quiet; Re gives nu_lbm = (tau - 0.5)/3.
    nu_lbm = (TAU - 0.5) / 3.0
    dt = (1.0 / n) / 16.0
    re = 1.0 / (nu_lbm * (1.0 / n) ** 2 / dt)
    d = hostcase.Definitions(dims=3, resolution=n, timestep=dt, bx=1.0, by=1.0, bz=nz / n, re=re,
                             walls=(A.FLUID,) * 6)
    l0 = hostcase.build_level0(d)
    l0.u = taylor_green(n, n, nz, U0, NOISE).reshape(-1)
    return l0


def equilibrium_f(l0):
    from luma_gb300 import case as hostcase
    return hostcase.equilibrium(3, 19, l0.rho, l0.u).reshape(-1)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.monotonic(), parts))

    def mark(self):
        return time.monotonic()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float) -> dict:
        inside = [p for (t, p) in self.samples if t0 - 0.15 <= t <= t1 + 0.15] or [p for (_, p) in self.samples]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(p[1]) for p in inside if num(p[1]) is not None]
        smax = [num(p[2]) for p in inside if num(p[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for p in inside for i in range(4) if p[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(inside),
                "power_w_max": max((num(p[3]) or 0.0) for p in inside)}


def read_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fp:
            d = json.load(fp)
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo), or ''."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as fp:
            for line in fp:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return ""


def read_profile_traffic(name: str):
    """Per-launch DRAM bytes from a committed ncu summary (profiles/<name>.txt,
    line 'dram_bytes_per_launch <bytes>'), or None."""
    p = os.path.join(ROOT, "profiles", name + ".txt")
    if not os.path.exists(p):
        return None
    with open(p) as fp:
        for line in fp:
            if line.startswith("dram_bytes_per_launch"):
                try:
                    return float(line.split()[1])
                except (IndexError, ValueError):
                    return None
    return None


class CpuBox:
    """The oracle (the reference's algorithm, FP64, bit-exact with its serial
    build) on the n x n x nz Taylor-Green box, for the CPU baseline."""

    def __init__(self, n: int, nz: int):
        from oracle import oracle as O
        self.O = O
        self.l0 = workload_level0(n, nz)
        self.g = O.OracleGrid(self.l0.desc())
        self.g.upload(equilibrium_f(self.l0), self.l0.u, self.l0.rho, None, 0)
        self.t = 0

    def time(self, steps: int, warmup: int, threads: int) -> dict:
        """Warm-up steps, then `steps` timed steps (wall clock) on `threads`
        host threads; the state carries on from the previous call."""
        used = self.O.set_threads(threads)
        if warmup:
            self.g.step(warmup)
        t0 = time.perf_counter()
        self.g.step(steps)
        dt = time.perf_counter() - t0
        self.t += warmup + steps
        return {"mlups": self.l0.ncell * steps / dt / 1e6, "threads": used, "seconds": dt, "steps": steps,
                "warmup": warmup}

    def close(self):
        self.g.close()


def cpu_baseline_full_box(n: int, steps_all: int = 4, steps_one: int = 3):
    """CPU baseline on the same n^3 box: all host threads (1 warm-up +
    steps_all timed), then 1 thread (1 warm-up + steps_one timed), fewer when
    a step would not fit the sample budget.  Returns (record, CpuBox at
    t = 1 + steps_all with the all-thread state saved as 'state')."""
    box = CpuBox(n, n)
    nth = os.cpu_count() or 1
    allt = box.time(steps_all, 1, nth)
    state = box.g.download()
    t_all = box.t
    est_one = allt["seconds"] / allt["steps"] * allt["threads"] * 1.3   # a 1-thread step, roughly
    k1 = max(1, min(steps_one, int(CPU_SAMPLE_BUDGET_S / max(est_one, 1e-3)) - 1))
    one = box.time(k1, 1, 1)
    box.O.set_threads(nth)
    rec = {"value": round(allt["mlups"], 3), "unit": "MLUPS", "cores": allt["threads"], "kind": "port",
           "same_config": True, "nproc": nth, "cpu_model": cpu_model(),
           "sample": f"{allt['steps']} LBM steps of the full {n}^3 box after 1 warm-up step, all "
                     f"{allt['threads']} host threads (oracle restatement of GridObj::LBM_multi_opt, FP64, "
                     f"bit-exact with the reference's serial build; OpenMP over the site loop), "
                     f"{allt['seconds']:.2f} s",
           "one_thread": {"value": round(one["mlups"], 3), "unit": "MLUPS", "cores": 1,
                          "sample": f"{one['steps']} LBM steps of the same box after 1 warm-up step, 1 thread, "
                                    f"{one['seconds']:.2f} s"}}
    return rec, box, state, t_all


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The largest of the ranks' values (the job's time is its slowest
    rank's); x itself without a process group."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mlups(world: int, sites_per_rank: int, steps: int, seconds: float) -> float:
    """Whole-job throughput of `world` replicas that each update
    sites_per_rank sites `steps` times, timed by the slowest rank."""
    return world * sites_per_rank * steps / seconds / 1e6


def run_reference(args, rank: int, world: int):
    """The reference's CPU path on the host cores: one LBM step of the full
    256^3 box per bench step on all host threads (a z-slab of the box per
    bench step only when K full-box steps would not fit the sample budget),
    then a 1-thread figure on the same box."""
    if rank != 0:
        return 0
    n = args.size or SIZE
    nth = os.cpu_count() or 1
    probe = CpuBox(n, n)
    est = probe.time(1, 0, nth)["seconds"]          # one full-box step
    nz = n
    if est * (args.steps + args.warmup) > CPU_SAMPLE_BUDGET_S:
        nz = max(8, int(n * CPU_SAMPLE_BUDGET_S / (est * (args.steps + args.warmup))) // 8 * 8)
    box = probe if nz == n else CpuBox(n, nz)
    if box is not probe:
        probe.close()
    allt = box.time(args.steps, args.warmup, nth)
    k1 = max(1, min(3, int(CPU_SAMPLE_BUDGET_S / max(est * nth * 1.3 * nz / n, 1e-3)) - 1))
    one = box.time(k1, 1, 1)
    box.close()
    mlups = allt["mlups"]
    what = f"the full {n}^3 box" if nz == n else f"a {n}x{n}x{nz} slab of the {n}^3 box"
    line = {
        "metric": METRIC, "value": round(mlups, 3), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(allt["seconds"] / args.steps * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": f"D3Q19 LBGK periodic {n}^3 Taylor-Green u0={U0} + U(-{NOISE},{NOISE}) noise "
                               f"(seed 20261203), tau={TAU}",
                   "precision": "fp64 (the reference's arithmetic)", "host_threads": allt["threads"],
                   "same_config": nz == n},
        "cpu_baseline": {"value": round(mlups, 3), "unit": "MLUPS", "cores": allt["threads"], "kind": "port",
                         "same_config": nz == n, "nproc": nth, "cpu_model": cpu_model(),
                         "sample": f"one LBM step of {what} per bench step, {args.steps} timed after "
                                   f"{args.warmup} warm-up (oracle restatement of GridObj::LBM_multi_opt, FP64, "
                                   f"bit-exact with the reference's serial build; OpenMP over the site loop)",
                         "one_thread": {"value": round(one["mlups"], 3), "unit": "MLUPS", "cores": 1,
                                        "sample": f"{one['steps']} LBM steps of {what} after 1 warm-up step, "
                                                  f"1 thread, {one['seconds']:.2f} s"}},
        "e2e": {"value": round(mlups, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_adjoint(nsteps: int = 4000, precisions=("fp32_shifted", "fp64")) -> dict:
    """Cost and memory of the drag gradient on the adjoint workload (D2Q9
    400x160 channel, IB cylinder of 64 markers, 4000 steps, checkpoints every
    100), FP32-shifted as the workload runs and FP64; wall clock around the
    C-ABI calls (each blocks until its result is on the host)."""
    from luma_gb300 import _abi as A
    from luma_gb300 import adjoint as ADJ

    c = ADJ.cylinder_channel(nsteps=nsteps)
    umax = ADJ.inlet_u_max(c)
    out = {"workload": "D2Q9 BGK channel 400x160, parabolic inlet u_max=0.05 lu, IB cylinder D=20 lu with 64 "
                       f"markers on radii 10+N(0,0.1^2) lu (seeded), {nsteps} steps, checkpoints every 100; "
                       "J = time-averaged drag; gradient w.r.t. u_max and 128 marker coordinates",
           "cost_definition": "(adjoint forward + backward) / plain forward (luma_gpu_step over the same steps), "
                       "for a repeated gradient on one grid; first_call_* includes the capture of the "
                       "segment graphs"}
    grads = {}
    for prec, name in ((A.PREC_FP32_SHIFTED, "fp32_shifted"), (A.PREC_FP64, "fp64")):
        if name not in precisions:
            continue
        warm = ADJ.DragCase(c.defs, c.markers, 200, 100)
        ADJ.drag_and_gradient(warm, prec)
        g, _ = ADJ.make_grid(c, prec)
        g.step(10)
        g.synchronize()
        t = time.perf_counter()
        g.step(c.nsteps)
        g.synchronize()
        plain = time.perf_counter() - t
        g.close()
        g, l0 = ADJ.make_grid(c, prec)
        _, f0, u0, rho0 = ADJ.initial_state(c.defs)
        force = l0.force_xyz.copy() if l0.force_xyz is not None else None
        calls = []
        # the first gradient on a grid captures the segment graphs; a repeat
        # from the same initial state (an optimisation loop's case) replays
        for _ in range(2):
            g.upload(f0, u0, rho0, force, t=0)
            g.synchronize()
            t = time.perf_counter()
            J = g.adj_forward(c.nsteps, c.checkpoint_every, 0)
            fwd = time.perf_counter() - t
            t = time.perf_counter()
            gs, gx = g.adj_backward(1.0)
            bwd = time.perf_counter() - t
            calls.append((fwd, bwd))
        mem = g.adj_memory()
        g.close()
        grads[name] = (gs, gx)
        first = sum(calls[0])
        out[name] = {"J": J, "dJ_du_max": gs / umax, "forward_s": round(fwd, 4), "backward_s": round(bwd, 4),
                     "plain_forward_s": round(plain, 4), "cost_vs_forward": round((fwd + bwd) / plain, 3),
                     "first_call_s": round(first, 4), "first_call_cost_vs_forward": round(first / plain, 3),
                     "backward_vs_adjoint_forward": round(bwd / fwd, 3), "device_bytes": int(mem)}
    if len(grads) == 2:
        g32, g64 = grads["fp32_shifted"], grads["fp64"]
        out["fp32_vs_fp64"] = {"dJ_ds_rel": abs(g32[0] - g64[0]) / abs(g64[0]),
                               "dJ_dX_rel_max": float(np.max(np.abs(g32[1] - g64[1])) / np.max(np.abs(g64[1])))}
    fdp = os.path.join(ROOT, "tests", "golden", "adjoint_fd_cyl400.json")
    if os.path.exists(fdp) and nsteps == 4000:
        ref = json.load(open(fdp))
        fd = np.array([r["fd"] for r in ref["markers"]])
        chk = {"source": "central differences of the reference's own FP64 build (h=1e-4)"}
        for name, (gs, gx) in grads.items():
            ad = np.array([gx[r["marker"], r["dim"]] for r in ref["markers"]])
            chk[name] = {"inlet_rel": abs(gs - ref["fd_inlet"]) / abs(ref["fd_inlet"]),
                         "markers_rel_max": float(np.max(np.abs(ad - fd)) / np.max(np.abs(fd)))}
        out["fd_check"] = chk
    return out


def trace_path(args, workload: str, prec: str) -> str | None:
    """Where --trace puts a workload's kernel timeline (a Chrome trace and
    its text summary beside it, written once the workload has run)."""
    if not args.trace:
        return None
    os.makedirs(args.trace, exist_ok=True)
    return os.path.join(args.trace, f"{workload}_{prec}_timeline.json")


def write_trace_summaries(args, workload: str, names) -> None:
    from luma_gb300 import timeline
    for name in names:
        p = trace_path(args, workload, name)
        if p and os.path.exists(p):
            with open(p[:-5] + ".txt", "w") as fh:
                fh.write(timeline.summarize(p, 4))


def run_sphere_workload(args) -> int:
    """D3Q19 flow past an IB sphere with two refinement levels (384x192x192
    base; ``--size`` scales the base x extent and everything with it):
    fine-weighted MLUPS, drag coefficient, FP32-vs-FP64 fields."""
    from luma_gb300 import _abi as A
    from luma_gb300 import workloads as WL

    nx = args.size or 384
    sc = nx / 384.0
    kw = dict(nx=nx, ny=nx // 2, nz=nx // 2, diameter_lu=24.0 * sc, n_markers=int(round(5000 * sc * sc)),
              l1_half=max(6, int(round(24 * sc))), l2_half=max(1, int(round(4 * sc))))
    res = {}
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    t0 = time.monotonic()
    for name, prec in (("fp32_shifted", A.PREC_FP32_SHIFTED), ("fp64", A.PREC_FP64)):
        if args.precision not in ("both", name.split("_")[0]):
            continue
        levels, markers = WL.sphere_refined(**kw)
        res[name] = WL.run_sphere(prec, args.steps, warmup=args.warmup, levels=levels, markers=markers,
                                  diameter_lu=kw["diameter_lu"], trace=trace_path(args, "sphere", name))
    t1 = time.monotonic()
    clocks = sampler.summary(t0, t1)
    head = res.get("fp32_shifted") or res.get("fp64")
    line = {"metric": "D3Q19 IBM sphere, two refinement levels: lattice updates per second (fine levels "
                      "counted 2^level times per base step)",
            "value": round(head["mlups"], 2), "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(head["ms_per_step"], 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if "fp32_shifted" in res else "f64",
            "data": "synthetic",
            "config": {"workload": f"D3Q19 LBGK {nx}x{nx // 2}x{nx // 2} base grid, level-1 box "
                                   f"+-{kw['l1_half']} and level-2 box +-{kw['l2_half']} base cells around the "
                                   f"sphere (D={kw['diameter_lu']:g} base lu, {kw['n_markers']} Fibonacci markers "
                                   f"on level 1), inlet u=0.04 lu, Re=100, lateral faces periodic",
                       "sites_per_level": head["sites"], "lattice_updates_per_base_step":
                           head["lattice_updates_per_step"]},
            "clocks": clocks}
    # every level carries a force field (IB grids): 2*Q*s populations + the
    # label byte + dims*s force bytes per lattice update, the step as a whole
    peaks = read_peaks()
    s_b = 4 if "fp32_shifted" in res else 8
    bpl = 2 * 19 * s_b + 1 + 3 * s_b
    line["roofline"] = {"bound": "hbm", "bytes_per_lu": bpl, "achieved": round(head["mlups"] * 1e6 * bpl / 1e9, 1),
                        "peak": peaks["hbm_gbs"], "unit": "GB/s",
                        "frac": round(head["mlups"] * 1e6 * bpl / 1e9 / peaks["hbm_gbs"], 4),
                        "note": "whole step (all kernels) against 2*Q*s+1+3*s bytes per lattice update, fine "
                                "levels counted 2^level times per base step"}
    for name, r in res.items():
        line[name] = {"mlups": round(r["mlups"], 2), "ms_per_step": round(r["ms_per_step"], 4), "cd": r["cd"],
                      "force": r["force"], "ibm_init_s": round(r["ibm_init_s"], 3)}
    if len(res) == 2:
        u32, u64 = res["fp32_shifted"]["u0"], res["fp64"]["u0"]
        r32, r64 = res["fp32_shifted"]["rho0"], res["fp64"]["rho0"]
        line["fp32_vs_fp64"] = {"rel_l2_u_level0": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
                                "max_abs_rho_level0": float(np.max(np.abs(r32 - r64))),
                                "cd_rel": abs(res["fp32_shifted"]["cd"] - res["fp64"]["cd"]) / abs(res["fp64"]["cd"]),
                                "speedup": round(res["fp32_shifted"]["mlups"] / res["fp64"]["mlups"], 3)}
    write_trace_summaries(args, "sphere", res)
    print(json.dumps(line), flush=True)
    return 0


def run_filaments_workload(args) -> int:
    """D3Q27 KBC (streamed-population form) 512x256x256 with one refinement
    level around 64 FEM filaments: MLUPS, HBM fraction, tip displacement of
    FP32 vs FP64 after the same steps."""
    from luma_gb300 import _abi as A
    from luma_gb300 import workloads as WL

    nx = args.size or 512
    sc = nx / 512.0
    kw = dict(nx=nx, ny=nx // 2, nz=nx // 2, box=(max(8, int(96 * sc)), max(8, int(64 * sc)), max(8, int(96 * sc))),
              resolution=max(4, int(32 * sc)), n_fil=64 if sc >= 0.5 else 4, nel=32 if sc >= 0.5 else 8)
    res = {}
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    t0 = time.monotonic()
    for name, prec in (("fp32_shifted", A.PREC_FP32_SHIFTED), ("fp64", A.PREC_FP64)):
        if args.precision not in ("both", name.split("_")[0]):
            continue
        levels, fils = WL.kbc_filaments(**kw)
        res[name] = WL.run_filaments(prec, args.steps, warmup=args.warmup, levels=levels, fils=fils,
                                     trace=trace_path(args, "filaments", name))
    t1 = time.monotonic()
    clocks = sampler.summary(t0, t1)
    peaks = read_peaks()
    head = res.get("fp32_shifted") or res.get("fp64")
    s = 4 if "fp32_shifted" in res else 8
    bpl = 2 * 27 * s + 1
    line = {"metric": "D3Q27 KBC + refinement + 64 FEM filaments: lattice updates per second (level 1 counted "
                      "twice per base step)",
            "value": round(head["mlups"], 2), "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(head["ms_per_step"], 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if s == 4 else "f64", "data": "synthetic",
            "config": {"workload": f"D3Q27 KBC (streamed-population form) {nx}x{nx // 2}x{nx // 2}, level-1 box "
                                   f"{kw['box']} base cells, {kw['n_fil']} filaments x {kw['nel']} elements "
                                   f"(one marker per node), EI log-uniform [1e-3,1e-1] (EI/(rho U^2 L^3)), "
                                   f"structure/fluid density 100, inlet u=0.03 lu, Re=1000 on the filament length",
                       "sites_per_level": head["sites"], "lattice_updates_per_base_step":
                           head["lattice_updates_per_step"]},
            "roofline": {"bound": "hbm", "bytes_per_lu": bpl,
                         "achieved": round(head["mlups"] * 1e6 * bpl / 1e9, 1), "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": round(head["mlups"] * 1e6 * bpl / 1e9 / peaks["hbm_gbs"], 4),
                         "note": "whole step (all kernels) against 2*Q*s+1 bytes per lattice update"},
            "clocks": clocks}
    for name, r in res.items():
        disp = r["tips"] - r["tip0"]
        line[name] = {"mlups": round(r["mlups"], 2), "ms_per_step": round(r["ms_per_step"], 4),
                      "finite": r["finite"], "ibm_init_s": round(r["ibm_init_s"], 3),
                      "tip_displacement_max": float(np.max(np.linalg.norm(disp, axis=1)))}
    if len(res) == 2:
        d32 = res["fp32_shifted"]["tips"] - res["fp32_shifted"]["tip0"]
        d64 = res["fp64"]["tips"] - res["fp64"]["tip0"]
        line["fp32_vs_fp64"] = {
            "tip_displacement_rel_err": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
            "rel_l2_u_level0": float(np.linalg.norm(res["fp32_shifted"]["u0"] - res["fp64"]["u0"]) /
                                     np.linalg.norm(res["fp64"]["u0"])),
            "speedup": round(res["fp32_shifted"]["mlups"] / res["fp64"]["mlups"], 3)}
    write_trace_summaries(args, "filaments", res)
    print(json.dumps(line), flush=True)
    return 0


def run_bfl_workload(args) -> int:
    """D2Q9 channel 8192x2048 with a BFL cylinder (radius 128 lu): MLUPS,
    HBM fraction of the whole step, body force, FP32 vs FP64; the oracle
    (serial on BFL grids) timed on a few steps of the same grid."""
    from luma_gb300 import _abi as A
    from luma_gb300 import workloads as WL

    nx = args.size or 8192
    kw = dict(nx=nx, ny=nx // 4, radius_lu=128.0 * nx / 8192.0)
    l0, body = WL.bfl_cylinder(**kw)
    res = {}
    sampler = ClockSampler(0)
    sampler.start()
    time.sleep(0.3)
    t0 = time.monotonic()
    for name, prec in (("fp32_shifted", A.PREC_FP32_SHIFTED), ("fp64", A.PREC_FP64)):
        if args.precision not in ("both", name.split("_")[0]):
            continue
        res[name] = WL.run_bfl(prec, args.steps, warmup=args.warmup, l0=l0, body=body)
    t1 = time.monotonic()
    clocks = sampler.summary(t0, t1)
    peaks = read_peaks()
    head = res.get("fp32_shifted") or res.get("fp64")
    s = 4 if "fp32_shifted" in res else 8
    bpl = 2 * 9 * s + 1
    line = {"metric": "D2Q9 channel with a BFL cylinder: lattice updates per second",
            "value": round(head["mlups"], 2), "unit": "MLUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(head["ms_per_step"], 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if s == 4 else "f64", "data": "synthetic",
            "config": {"workload": f"D2Q9 LBGK {l0.N}x{l0.M}, solid bottom/top, uniform forced-equilibrium inlet "
                                   f"u=0.04 lu, extrapolate-right outlet, BFL cylinder radius {kw['radius_lu']:g} lu "
                                   f"(CIRCLE_SPHERE BFL prefab, {head['markers']} markers, {head['links']} wall "
                                   f"links), Re_D=250", "inputs": "larger than L2"},
            "roofline": {"bound": "hbm", "bytes_per_lu": bpl,
                         "achieved": round(head["mlups"] * 1e6 * bpl / 1e9, 1), "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": round(head["mlups"] * 1e6 * bpl / 1e9 / peaks["hbm_gbs"], 4),
                         "note": "whole step (all kernels) against 2*Q*s+1 bytes per lattice update"},
            "clocks": clocks}
    for name, r in res.items():
        line[name] = {"mlups": round(r["mlups"], 2), "ms_per_step": round(r["ms_per_step"], 4),
                      "body_force": r["force"]}
    if len(res) == 2:
        u32, u64 = res["fp32_shifted"]["u"], res["fp64"]["u"]
        f32, f64 = res["fp32_shifted"]["force"][0], res["fp64"]["force"][0]
        line["fp32_vs_fp64"] = {"rel_l2_u": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
                                "drag_rel": abs(f32 - f64) / abs(f64),
                                "speedup": round(res["fp32_shifted"]["mlups"] / res["fp64"]["mlups"], 3)}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        from luma_gb300 import case as hostcase
        o = O.OracleGrid(l0.desc())
        o.upload(hostcase.equilibrium(2, 9, l0.rho, l0.u).reshape(-1), l0.u, l0.rho, None, 0)
        o.bfl_set(body.site_marker, body.q)
        o.step(1)
        nst = 2
        t = time.perf_counter()
        o.step(nst)
        dt = time.perf_counter() - t
        line["cpu_baseline"] = {"value": round(l0.ncell * nst / dt / 1e6, 2), "unit": "MLUPS", "cores": 1,
                                "kind": "port", "sample": f"{nst} steps of the same grid on the oracle (FP64; "
                                                          f"serial: BFL marker forces accumulate in site order), "
                                                          f"{dt:.1f} s"}
        o.close()
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank: int, world: int, local_rank: int):
    import torch
    from luma_gb300 import _abi as A
    from luma_gb300.gpu import GpuGrid

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist_
        dist_.init_process_group("nccl")
        dist = dist_
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    n = args.size or SIZE
    l0 = workload_level0(n)
    f0 = equilibrium_f(l0)
    ncell = l0.ncell
    K, W = args.steps, args.warmup

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks_(x: float) -> float:
        return max_over_ranks(x, dist, dev)

    def warm(grid, steps):
        # One single step, then the rest in one call: that call captures the
        # two-step CUDA graph at the storage parity the timed call starts
        # from (steps - 1 >= 4 steps) and runs its last steps directly, so
        # every kernel and graph the timed call uses is loaded and captured
        # before the timed region.
        grid.step(1)
        grid.step(steps - 1)

    def timed_steps(grid, steps, sampler=None):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        t0 = time.monotonic()
        e0.record(stream)
        grid.step(steps)
        e1.record(stream)
        e1.synchronize()
        t1 = time.monotonic()
        barrier()
        return e0.elapsed_time(e1) / 1e3, t0, t1

    # ---- FP32 shifted (headline) ----
    g32 = GpuGrid(l0.desc(precision=A.PREC_FP32_SHIFTED))
    g32.set_stream(stream.cuda_stream)
    g32.upload(f0, l0.u, l0.rho, None, 0)
    warm(g32, W)
    sampler = ClockSampler(local_rank if "CUDA_VISIBLE_DEVICES" not in os.environ else 0)
    sampler.start()
    time.sleep(0.3)
    sec32, t0, t1 = timed_steps(g32, K)
    sampler_summary = sampler.summary(t0, t1)
    sec32 = max_over_ranks_(sec32)
    mlups32 = replica_mlups(world, ncell, K, sec32)
    g32.synchronize()

    # ---- FP64 (the reference's arithmetic) on the same workload ----
    K64 = min(K, max(K // 4, 20))
    g64 = GpuGrid(l0.desc(precision=A.PREC_FP64))
    g64.set_stream(stream.cuda_stream)
    g64.upload(f0, l0.u, l0.rho, None, 0)
    warm(g64, W)
    sec64, _, _ = timed_steps(g64, K64)
    sampler.stop()
    sec64 = max_over_ranks_(sec64)
    mlups64 = replica_mlups(world, ncell, K64, sec64)
    # accuracy at equal step counts, outside the timed regions: both paths
    # to t = 10^4 (or W + K when the timed run went further)
    t_acc = max(ACCURACY_STEPS, W + K)
    g32.step(t_acc - g32.t)
    g64.step(t_acc - g64.t)
    g32.synchronize()
    g64.synchronize()
    s32 = g32.download(f=False)
    s64 = g64.download(f=False)
    eu = float(np.linalg.norm(s32["u"] - s64["u"]) / np.linalg.norm(s64["u"]))
    er = float(np.linalg.norm(s32["rho"] - s64["rho"]) / np.linalg.norm(s64["rho"]))
    red64 = g64.reduce()
    red32 = g32.reduce()
    g64.close()

    # ---- e2e through the C ABI with host buffers (pinned) ----
    import torch as _t
    hf = _t.from_numpy(f0).pin_memory()
    hu = _t.from_numpy(l0.u).pin_memory()
    hr = _t.from_numpy(l0.rho).pin_memory()
    out_u = _t.empty(ncell * 3, dtype=_t.float64).pin_memory()
    out_r = _t.empty(ncell, dtype=_t.float64).pin_memory()
    import ctypes as C
    from luma_gb300.gpu import check, lib
    L = lib()
    dp = C.POINTER(C.c_double)
    ptr = lambda t: C.cast(t.data_ptr(), dp)  # noqa: E731
    # warm the pool and the paths (graph capture included) with one untimed
    # run of the same calls
    check(L.luma_gpu_upload_state(C.c_void_p(g32.h), ptr(hf), ptr(hu), ptr(hr), None, 0))
    check(L.luma_gpu_step(C.c_void_p(g32.h), K))
    check(L.luma_gpu_download_state(C.c_void_p(g32.h), None, ptr(out_u), ptr(out_r), None))
    barrier()
    runs = []
    for _ in range(3):   # the whole-call time varies with the host link; the median is reported
        t_e0 = time.perf_counter()
        check(L.luma_gpu_upload_state(C.c_void_p(g32.h), ptr(hf), ptr(hu), ptr(hr), None, 0))
        check(L.luma_gpu_step(C.c_void_p(g32.h), K))
        check(L.luma_gpu_download_state(C.c_void_p(g32.h), None, ptr(out_u), ptr(out_r), None))
        barrier()
        runs.append(max_over_ranks_(time.perf_counter() - t_e0))
    sec_e2e = sorted(runs)[1]
    e2e = replica_mlups(world, ncell, K, sec_e2e)
    h2d = (f0.nbytes + l0.u.nbytes + l0.rho.nbytes) / K
    d2h = (out_u.numel() + out_r.numel()) * 8 / K
    # one more call, its phases timed apart (each call blocks or is followed by a sync)
    t_a = time.perf_counter()
    check(L.luma_gpu_upload_state(C.c_void_p(g32.h), ptr(hf), ptr(hu), ptr(hr), None, 0))
    t_b = time.perf_counter()
    check(L.luma_gpu_step(C.c_void_p(g32.h), K))
    check(L.luma_gpu_synchronize(C.c_void_p(g32.h)))
    t_c = time.perf_counter()
    check(L.luma_gpu_download_state(C.c_void_p(g32.h), None, ptr(out_u), ptr(out_r), None))
    t_d = time.perf_counter()
    e2e_phases = {"upload_s": round(t_b - t_a, 5), "steps_s": round(t_c - t_b, 5), "download_s": round(t_d - t_c, 5),
                  "upload_gbs": round((f0.nbytes + l0.u.nbytes + l0.rho.nbytes) / (t_b - t_a) / 1e9, 1),
                  "download_gbs": round((out_u.numel() + out_r.numel()) * 8 / (t_d - t_c) / 1e9, 1)}
    g32.close()

    # ---- roofline ----
    peaks = read_peaks()
    bytes32 = 2 * 19 * 4 * ncell
    ach32 = bytes32 / (sec32 / K) / 1e9
    traffic = read_profile_traffic("k_aa_d3q19_fp32_256") if n == SIZE else None
    bytes64 = 2 * 19 * 8 * ncell

    adjoint = measure_adjoint() if rank == 0 and not args.no_adjoint else None

    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, box, ostate, t_o = cpu_baseline_full_box(n, steps_all=args.cpu_steps)
        # the FP64 GPU path at full size against the CPU leg's own state (the
        # oracle after the same steps from the same initial state)
        gp = GpuGrid(l0.desc(precision=A.PREC_FP64))
        gp.set_stream(stream.cuda_stream)
        gp.upload(f0, l0.u, l0.rho, None, 0)
        gp.step(t_o)
        gs = gp.download()
        gp.close()
        box.close()
        rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
        parity = {"after_steps": t_o, "rel_l2_u": rl(gs["u"], ostate["u"]), "rel_l2_rho": rl(gs["rho"], ostate["rho"]),
                  "rel_l2_f": rl(gs["f"], ostate["f"]), "bound": 1e-10,
                  "what": f"GPU FP64 path vs the oracle (the reference's arithmetic) on the full {n}^3 box"}
        del gs, ostate

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(mlups32, 2), "unit": "MLUPS", "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": round(sec32 / K * 1e3, 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"D3Q19 LBGK periodic {n}^3 Taylor-Green u0={U0} + U(-{NOISE},{NOISE}) noise "
                                   f"(seed 20261203), tau={TAU}",
                       "precision": "fp32_shifted (f_i - w_i*rho0 stored in FP32, FP32 collision)",
                       "streaming": "in-place AA pattern, SoA", "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1.27 GB FP32 populations per grid)"},
            "clocks": sampler_summary,
            "e2e": {"value": round(e2e, 2), "unit": "MLUPS", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "note": "C ABI with pinned host buffers (read and written in place by the layout "
                            "conversions): upload of FP64 reference-layout state, K steps, download of u and "
                            "rho; median of 3 timed calls",
                    "calls_s": [round(x, 5) for x in runs], "phases": e2e_phases},
            "gpu_launches": K,
            "roofline": {"bound": "hbm", "achieved": round(ach32, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": round(ach32 / peaks["hbm_gbs"], 4), "traffic": traffic,
                         "traffic_source": ("profiles/k_aa_d3q19_fp32_256.txt: dram__bytes_read.sum + "
                                            "dram__bytes_write.sum of one launch of this kernel on this workload "
                                            "(ncu, 1 pass), not measured in this run") if traffic else None,
                         "peak_source": peaks["source"], "kernel": "k_aa<19,P32>",
                         "bytes_per_launch": bytes32},
            "fp64": {"value": round(mlups64, 2), "unit": "MLUPS", "steps": K64,
                     "ms_per_step": round(sec64 / K64 * 1e3, 4),
                     "hbm_gbs": round(bytes64 / (sec64 / K64) / 1e9, 1),
                     "hbm_frac": round(bytes64 / (sec64 / K64) / 1e9 / peaks["hbm_gbs"], 4),
                     "fp64_tflops": round(mlups64 * 1e6 * FP64_FLOP_PER_LU_D3Q19 / 1e12, 3),
                     "fp64_frac_of_nominal": round(mlups64 * 1e6 * FP64_FLOP_PER_LU_D3Q19 / 1e12 /
                                                   FP64_NOMINAL_TFLOPS, 3),
                     "bound": "FP64 pipe (231 FP64 FLOP per update, counted with ncu)"},
            "fp32_vs_fp64": {"speedup": round(mlups32 / mlups64, 3), "rel_l2_u": eu, "rel_l2_rho": er,
                             "after_steps": t_acc, "bound_rel_l2_u": 1e-5, "fp64_mass": red64["mass"],
                             "fp32_mass": red32["mass"],
                             "what": "both paths from the same initial state to t = after_steps (untimed)"},
            "fp64_parity_full_size": parity,
            "cpu_baseline": cpu,
            "adjoint": adjoint,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=None,
                    help="box edge (default 256) or, for --workload sphere, base x extent (default 384)")
    ap.add_argument("--workload", default="box", choices=["box", "sphere", "cylinder_adjoint", "filaments", "bfl"],
                    help="box: the headline 256^3 line (default); sphere: IB sphere with two refinement "
                         "levels; cylinder_adjoint: the drag-gradient workload alone; filaments: D3Q27 KBC with "
                         "one refinement level and 64 FEM filaments; bfl: D2Q9 channel with a BFL cylinder")
    ap.add_argument("--precision", default="both", choices=["both", "fp32", "fp64"],
                    help="sphere / cylinder_adjoint workloads: which precisions to run")
    ap.add_argument("--cpu-steps", type=int, default=4, help="timed all-thread steps of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint workload measurement")
    ap.add_argument("--trace", default=None, metavar="DIR",
                    help="sphere/filaments: after the measurement, record 4 more steps as a kernel timeline "
                         "(CUPTI through torch.profiler) into DIR, with a text summary")
    args = ap.parse_args(argv)
    if args.warmup < 5:
        args.warmup = 5     # the headline warm-up captures its step graph in >= 4 steps after one
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "sphere":
        return run_sphere_workload(args) if rank == 0 else 0
    if args.workload == "filaments":
        return run_filaments_workload(args) if rank == 0 else 0
    if args.workload == "bfl":
        return run_bfl_workload(args) if rank == 0 else 0
    if args.workload == "cylinder_adjoint":
        if rank == 0:
            prec = {"both": ("fp32_shifted", "fp64"), "fp32": ("fp32_shifted",), "fp64": ("fp64",)}[args.precision]
            steps = args.steps if args.steps != 2000 else 4000
            print(json.dumps({"workload": "cylinder_adjoint", "adjoint": measure_adjoint(steps, prec)}), flush=True)
        return 0
    return run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    sys.exit(main())
