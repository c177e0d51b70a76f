"""Multi-GPU host logic on CPU: world_size 2 over gloo.

The path runs as independent replicas (no exchange step); the only
cross-rank operations are the barrier and the max-over-ranks time that
bench.py uses for the whole-job throughput.
"""

from __future__ import annotations

import os
import socket

import pytest

from glass_gb300 import replicas


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, queue) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    replicas.init("gloo")
    assert replicas.dist_env() == (rank, world, rank)
    replicas.barrier()
    # rank r "took" 1.5 + r seconds for 3 steps of 10 units
    slowest = replicas.max_over_ranks(1.5 + rank)
    value = replicas.replica_throughput(world, 10.0, 3, slowest)
    replicas.barrier()
    replicas.shutdown()
    queue.put((rank, slowest, value))


def test_max_over_ranks_and_throughput_world2():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(queue.get(timeout=10) for _ in range(2))
    for rank, slowest, value in results:
        assert slowest == 2.5
        assert value == pytest.approx(2 * 10.0 * 3 / 2.5)


def test_single_process_defaults():
    assert replicas.max_over_ranks(4.0) == 4.0
    assert replicas.replica_throughput(1, 5.0, 2, 2.0) == 5.0
    with pytest.raises(ValueError):
        replicas.replica_throughput(1, 5.0, 2, 0.0)
