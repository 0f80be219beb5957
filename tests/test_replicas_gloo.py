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


def _shard_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        lo, hi = bench.shard(2048, rank, world)
        # each rank "runs" its graphs: edges = the sum of its graph ids, time = its graph count
        edges = sum(range(lo, hi))
        q.put((rank, (lo, hi), bench.job_reduce(dist, float(hi - lo), edges, None)))
    finally:
        dist.destroy_process_group()


def test_sharded_batch_two_ranks():
    """The batched section's N > 1 path: each rank takes a contiguous share
    of the 2,048-graph work queue; the job time is the slowest rank's and the
    job's edges are every rank's, gathered on the host side."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        rank, rng, red = q.get(timeout=120)
        out[rank] = (rng, red)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] == (0, 1024) and out[1][0] == (1024, 2048)
    for r in (0, 1):
        ms, edges = out[r][1]
        assert ms == 1024.0 and edges == float(sum(range(2048)))


def test_shard_covers_every_unit_once():
    import bench

    for n in (0, 1, 7, 256, 2048):
        for world in (1, 2, 3, 8):
            parts = [bench.shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
