"""bench.py's multi-rank host logic (replicas: slowest rank's time, summed
lattice updates) on world_size-2 gloo process groups on the CPU."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_env() == (ws, rank, rank)
        ms = bench.slowest_rank_ms(1.5 + rank, ws, "cpu")   # rank 1 is the slow one
        out.put((rank, ms, bench.job_mlups(1000, ms, ws)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_slowest_rank_and_job_throughput_gloo():
    torch = pytest.importorskip("torch")
    import socket
    mp = torch.multiprocessing.get_context("spawn")
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    q = mp.Queue()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, mlups in res:
        assert ms == 2.5                      # the slowest rank's time on every rank
        assert abs(mlups - 1000 * 2 / 2500) < 1e-12   # both replicas' updates in that time


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.slowest_rank_ms(3.25, 1) == 3.25
    assert bench.job_mlups(1000, 2.0, 1) == 0.5


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    """Under torchrun the reference arm runs on rank 0 only; the other ranks
    return 0 at once (no oracle build, no output)."""
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(argparse.Namespace(steps=3, warmup=3, gpus=2)) == 0


def test_trimmed_mean_is_benchmark_sh():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.trimmed_mean([5.0, 1.0, 3.0, 9.0, 4.0]) == 4.0   # drops 1 and 9
    assert bench.trimmed_mean([2.0, 2.0, 2.0]) == 2.0
    with pytest.raises(ValueError):
        bench.trimmed_mean([1.0, 2.0])
