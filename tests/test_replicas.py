"""The multi-process path of bench.py on CPU (gloo, world size 2): every
configuration fits one GB300, so N GPUs run N independent replicas and the
job's time per step is the slowest replica's (all-reduce MAX); the CPU
reference arm prints from rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        got = bench.max_over_ranks(10.0 + 5.0 * rank, dist)      # rank 1 is the slow replica
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get() for _ in range(world))
    assert got == {0: 15.0, 1: 15.0}


def test_max_over_ranks_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5


def test_reference_arm_prints_on_rank0_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(bench.parse(["--impl", "reference"]))
    assert buf.getvalue() == ""


def test_bench_reads_committed_traffic():
    """The roofline's DRAM traffic comes from the committed ncu summary."""
    sys.path.insert(0, ROOT)
    import bench
    for kind in ("ilu_apply", "spmv", "euler_ebemv", "euler_ebemv32"):
        v = bench.read_traffic(kind)
        assert v is not None and v > 1e7, kind
    assert bench.read_traffic("no such kernel") is None
