"""bench.py's multi-rank logic on CPU: two gloo ranks (replicas only, no
data-path collective) agree on the slowest rank's time, the job value counts
every replica, and the reference arm does its work on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup()
        assert (w, r, local) == (world, rank, rank)
        t = bench.reduce_max(100.0 + 10.0 * rank, w)         # ms of this rank's steps
        v = bench.job_value(w, 1 << 21, 5, t)

        class A:
            warmup, steps, gpus = 1, 1, world
        rc = bench.run_reference(A) if rank != 0 else 0    # rank != 0: no work, exit 0
        out[rank] = (t, v, rc)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, start_method="spawn")
    for rank in range(world):
        t, v, rc = out[rank]
        assert t == 110.0                                   # the slowest rank
        assert v == pytest.approx(2 * (1 << 21) * 5 / 0.110)
        assert rc == 0
