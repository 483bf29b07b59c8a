"""The bench's multi-GPU form is independent replicas (one process per GPU, no data-path
collective): the host-side barrier and max-over-ranks timing it uses are checked here
with two gloo ranks on the CPU, and so is the whole-job throughput they feed."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    d = bench.Dist()
    d.barrier()
    # each replica's timed total (ms); the job's time is the slowest replica's
    total = d.max(100.0 + 25.0 * rank)
    d.barrier()
    q.put((rank, d.world, total, bench.replica_throughput(d.world, 10, total)))
    d.close()


def test_two_replicas_barrier_and_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for _, world, total, value in out:
        assert world == 2
        assert total == 125.0  # the slower replica
        assert value == pytest.approx(2 * 10 / 0.125)  # all replicas' builds over the slowest time


def test_single_process_needs_no_process_group():
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        assert k not in os.environ or os.environ[k] in ("0", "1")
    d = bench.Dist()
    assert d.world == 1 and d.max(3.5) == 3.5
    d.barrier()
    d.close()
    assert bench.replica_throughput(1, 20, 200.0) == pytest.approx(100.0)
