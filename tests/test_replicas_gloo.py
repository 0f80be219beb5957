"""The N > 1 bench path on CPU: world_size 2 over gloo (127.0.0.1). Replicas
run the whole workload each; the job time is the slowest rank's, and the job
value counts every rank's edges. No data-path collective exists: the only
collective is the max over ranks of the step time."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms = [40.0, 50.0][rank]
        q.put((rank, bench.reduce_over_ranks(dist, ms, 1_000_000_000, None)))
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms, gteps = out[r]
        assert ms == 50.0  # the slowest rank
        assert gteps == pytest.approx(2 * 1e9 / 0.05 / 1e9)


def test_reduce_over_ranks_single_process():
    import bench

    assert bench.reduce_over_ranks(None, 20.0, 4e9) == (20.0, pytest.approx(200.0))
