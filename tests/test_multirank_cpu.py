"""The N-GPU path of bench.py on the host: two gloo ranks (world size 2).

bench.py runs one independent replica per GPU (the step has no data
exchange on one grid per GPU); the job's time is the slowest rank's and its
throughput counts every replica's updates.  These tests run the rank logic
with the gloo backend on CPU: the max-over-ranks reduction, the whole-job
throughput, and the reference arm printing from rank 0 only.
"""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local = [1.5, 2.5][rank]                      # each rank's timed seconds
    slowest = bench.max_over_ranks(local, dist, "cpu")
    value = bench.replica_mlups(world, 1000, 10, slowest)
    buf = io.StringIO()

    class Args:
        steps, warmup = 1, 3
    with redirect_stdout(buf):
        rc = bench.run_reference(Args, rank, world) if rank == 1 else 0
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fp:
        json.dump({"slowest": slowest, "value": value, "ref_rc": rc, "ref_out": buf.getvalue()}, fp)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_replica_accounting(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    r = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(world)]
    # every rank sees the slowest rank's time
    assert r[0]["slowest"] == r[1]["slowest"] == 2.5
    # whole-job throughput: world replicas x sites x steps / slowest time
    assert r[0]["value"] == pytest.approx(2 * 1000 * 10 / 2.5 / 1e6)
    # the reference arm: ranks other than 0 exit 0 without work or output
    assert r[1]["ref_rc"] == 0 and r[1]["ref_out"] == ""
