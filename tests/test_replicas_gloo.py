"""CPU, world size 2 over gloo: the replica aggregation bench.py uses for N > 1 GPUs.

Every rank runs an independent replica; the only exchange is a max-reduction of the per-step
times, and the job throughput counts the steps of all ranks.
"""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local = [10.0 + 5.0 * rank, 20.0 - 3.0 * rank]  # per-step ms of (mixed, fp64) on this replica
    ms, value = bench.aggregate_replicas(local, world=world, device="cpu")
    dist.barrier()
    queue.put((rank, ms, value))
    dist.destroy_process_group()


def test_replica_aggregation_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in results:
        assert ms == [15.0, 20.0]  # max over ranks, per quantity
        assert value == pytest.approx(2 * 1000.0 / 15.0)


def test_single_rank_needs_no_process_group():
    import bench

    ms, value = bench.aggregate_replicas([4.0, 8.0], world=1)
    assert ms == [4.0, 8.0] and value == pytest.approx(250.0)
