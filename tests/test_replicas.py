"""The N > 1 path of bench.py: one process per GPU, independent replicas of the path
(no data exchange; a view's pixels never leave its GPU), a barrier around the timed
region and the slowest rank's time. Run here as two gloo ranks on the CPU."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, seconds, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE=str(world), HL_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist

    w, r, _ = bench.dist_setup(world)
    assert (w, r) == (world, rank)
    bench.barrier(w)
    value, t = bench.replica_throughput(w, 1920 * 1080, 10, seconds[rank])
    out.put((rank, value, t))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_replicas_report_all_pixels_over_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    seconds = [0.010, 0.020]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, seconds, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    want = 2 * 10 * 1920 * 1080 / 0.020 / 1e6
    for rank, value, t in got:
        assert t == pytest.approx(0.020)
        assert value == pytest.approx(want)


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        steps, warmup, gpus = 1, 0, 2

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args, 2, 1)
    assert buf.getvalue() == ""
