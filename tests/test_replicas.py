"""The N > 1 path of bench.py on the CPU: one process per rank over gloo, as
torchrun launches it.  Each rank solves its own copy of the model (replicas, no
collective on the data path); the host barrier and the max over ranks around the
timed region are what ranks share."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out) -> None:
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist = bench.Dist(world)
    dist.barrier()
    out.put((rank, dist.max(10.0 * (rank + 1)), bench.dist_env()))
    dist.barrier()
    dist.close()


def test_barrier_and_max_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    port, world = _free_port(), 2
    queue = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in results] == [0, 1]
    assert all(m == 20.0 for _, m, _ in results)  # every rank sees the slowest rank's time
    assert [env for _, _, env in results] == [(2, 0, 0), (2, 1, 1)]


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the reference arm's work and line come from rank 0; other
    ranks return at once with status 0."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        scale = 1

    assert bench.run_reference(Args()) == 0
