"""Replica (multi-GPU) logic of bench.py with world-size-2 gloo ranks on the
CPU: the path does not shard, N GPUs run N independent chain sets, the job's
time is the slowest rank's and its throughput all ranks' units over that time;
only rank 0 prints."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    t = bench.max_over_ranks(ms, dist, "cpu")
    value = bench.aggregate(1000, world, t)
    seeds = [None] * world
    dist.all_gather_object(seeds, bench.replica_seed(20261203, rank))
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, t, value, seeds))


def test_max_over_ranks_and_aggregate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, value, seeds in res:
        assert t == 150.0  # every rank sees the slowest rank's time
        assert value == pytest.approx(2 * 1000 / 0.150)
        assert len(set(seeds)) == 2  # independent replicas


def test_only_rank0_reports(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.argparse.Namespace(workload="batched384_adj_f32", steps=1, warmup=3, gpus=2, serve_rate=20.0,
                                    serve_window=30.0)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""
