"""Multi-GPU form of the bench: replicas (one independent proof stream per
rank, no data-path collective). Covered on CPU with gloo: per-rank workloads
differ, and the job time is the maximum over ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    sys.path.insert(0, ROOT)
    import bench

    return bench


def test_rank_workloads_are_distinct_and_seeded():
    bench = _bench()
    pairs = [bench.workload(r) for r in range(8)]
    assert len(set(pairs)) == 8
    assert pairs[0] == bench.workload(0)  # deterministic from the seed
    assert all(0 <= a < bench.P and 0 <= b < bench.P for a, b in pairs)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    dev_ms, wall_s = 10.0 + 5.0 * rank, 0.02 + 0.01 * (world - 1 - rank)
    got = bench.aggregate_replicas(dist, dev_ms, wall_s, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_replica_time_is_the_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    world, port = 2, _free_port()
    q = mp.Queue()
    procs = [mp.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in range(world):
        dev_ms, wall_s = res[rank]
        assert dev_ms == pytest.approx(15.0) and wall_s == pytest.approx(0.03)
