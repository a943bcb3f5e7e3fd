"""The N > 1 path of bench.py (independent replicas) as world_size-2 gloo
process groups on the CPU: the step time is the slowest rank's on every rank,
and the reference arm runs on rank 0 alone."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        args = bench.argparse.Namespace(ref_n=10, ref_gates=2, seed=3, warmup=1, steps=1)
        buf = io.StringIO()
        with redirect_stdout(buf):
            bench.run_reference(args, rank, world)
        dist.barrier()
        q.put((rank, ms, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_reference_runs_on_rank0():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(world):
        rank, ms, text = q.get(timeout=120)
        out[rank] = (ms, text)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 15.0
    assert '"impl": "reference"' in out[0][1] and out[1][1] == ""
