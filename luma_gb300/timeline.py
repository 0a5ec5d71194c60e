"""Kernel timeline of a few steps: start, duration and stream of every kernel
the library launches, including the kernels of replayed step graphs, from
CUPTI activity records (through torch.profiler).  An ncu launch list runs
the kernels one at a time; this shows how the streams of a step overlap
(the sub-grids' chain beside the base grid's interior, the listed sites
beside the interior) and which chain sets the step's length.  Taken after
a timed region, never inside one."""
from __future__ import annotations

import collections
import json
import re


def record(grid0, steps: int, path: str) -> None:
    """Steps the tree of `grid0` `steps` times under the profiler and writes
    the Chrome trace to `path`."""
    import torch
    from torch.profiler import ProfilerActivity, profile

    # the first profiling session of a process can come back without kernel
    # records: a short throwaway session first
    x = torch.zeros(1 << 16, device="cuda")
    with profile(activities=[ProfilerActivity.CUDA]):
        x.add_(1.0)
        torch.cuda.synchronize()
    grid0.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        grid0.step(steps)
        grid0.synchronize()
    prof.export_chrome_trace(path)


def _name(e: dict) -> str:
    n = re.sub(r"void |luma::|\(anonymous namespace\)::", "", e["name"])
    return n.split("(")[0]


def summarize(path: str, steps: int) -> str:
    """Per (kernel, stream): launches and device time per step, mean time
    per launch; the span per step and the busiest stream's share of it."""
    ev = json.load(open(path))
    ev = ev["traceEvents"] if isinstance(ev, dict) else ev
    k = sorted((e for e in ev if e.get("cat") == "kernel"), key=lambda e: e["ts"])
    if not k:
        return "no kernel records\n"
    t0 = k[0]["ts"]
    t1 = max(e["ts"] + e["dur"] for e in k)
    agg = collections.defaultdict(lambda: [0, 0.0])
    per_stream = collections.defaultdict(float)
    for e in k:
        s = e["args"].get("stream", -1)
        a = agg[(_name(e), s)]
        a[0] += 1
        a[1] += e["dur"]
        per_stream[s] += e["dur"]
    span = (t1 - t0) / steps
    lines = [f"{len(k)} kernels over {steps} steps; span {span:.1f} us per step"]
    for s, t in sorted(per_stream.items(), key=lambda x: -x[1]):
        lines.append(f"  stream {s}: kernels busy {t / steps:.1f} us per step ({100 * t / steps / span:.0f}% of the span)")
    lines.append(f"{'kernel':46s} {'stream':>6s} {'n/step':>7s} {'us/step':>9s} {'us/launch':>10s}")
    for (n, s), (c, t) in sorted(agg.items(), key=lambda x: -x[1][1]):
        lines.append(f"{n[:46]:46s} {s:6d} {c / steps:7.1f} {t / steps:9.1f} {t / c:10.1f}")
    return "\n".join(lines) + "\n"
