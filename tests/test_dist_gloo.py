"""bench.py's multi-process plumbing on CPU: world_size 2 over gloo.

Each process of this project drives one GPU, so N > 1 runs are replicas of the
single-GPU step (one process per GPU, no collective on the data path); what
they share is the barrier and the max-over-ranks of the timed region, tested
here with two CPU processes.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        m = d.max(1.5 + rank)          # the slowest rank's time
        args = bench.parse(["--impl", "reference", "--steps", "1", "--warmup", "0"])
        rec = bench.run_reference(args, d) if rank != 0 else "skipped"
        q.put((rank, d.world, m, rec))
    finally:
        d.close()


def test_two_ranks_share_barrier_and_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2, 2]
    assert [o[2] for o in out] == [2.5, 2.5]      # max over ranks on every rank
    assert out[1][3] is None                      # reference arm: rank 1 does no work
