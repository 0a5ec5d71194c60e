"""luma_gb300.timeline.summarize on a small synthetic Chrome trace: per
(kernel, stream) launches and time per step, the span per step and each
stream's busy share."""
import json

from luma_gb300 import timeline


def test_summary_of_two_streams(tmp_path):
    ev = [{"ph": "X", "cat": "kernel", "name": "void luma::(anonymous namespace)::k_interior<19, luma::P32>(x)",
           "ts": 1000.0 + 100.0 * s, "dur": 80.0, "args": {"stream": 7}} for s in range(2)]
    ev += [{"ph": "X", "cat": "kernel", "name": "void luma::k_ibm_spread<19, luma::P32>(y)",
            "ts": 1010.0 + 100.0 * s, "dur": 20.0, "args": {"stream": 15}} for s in range(2)]
    ev.append({"ph": "X", "cat": "cuda_runtime", "name": "cudaGraphLaunch", "ts": 990.0, "dur": 5.0})
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"traceEvents": ev}))
    out = timeline.summarize(str(p), 2)
    lines = out.splitlines()
    assert lines[0] == "4 kernels over 2 steps; span 90.0 us per step"
    assert "stream 7: kernels busy 80.0 us per step (89% of the span)" in out
    assert "stream 15: kernels busy 20.0 us per step (22% of the span)" in out
    row = [l for l in lines if l.startswith("k_interior<19, P32>")][0].split()
    assert row[-4:] == ["7", "1.0", "80.0", "80.0"]


def test_summary_without_kernels(tmp_path):
    p = tmp_path / "t.json"
    p.write_text(json.dumps({"traceEvents": []}))
    assert timeline.summarize(str(p), 4) == "no kernel records\n"
