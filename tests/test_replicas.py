"""Multi-GPU = replicas: every rank runs its own realisations (seed per rank and
step), the job's time is the slowest rank's, and the whole-job rate counts every
rank's units.  The aggregation runs here on two gloo ranks on the CPU; the
reference arm leaves every rank but 0 idle."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    ms = [100.0, 130.0][rank]
    slowest = bench.max_over_ranks(ms, ws, device="cpu")
    rate = bench.whole_job_rate(1024 ** 3, 4, ws, slowest)
    seeds = [bench.replica_seed(3001, rank, i) for i in range(4)]
    gathered = [None] * ws
    dist.all_gather_object(gathered, seeds)
    q.put((rank, slowest, rate, gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate, gathered in results:
        assert slowest == 130.0
        assert rate == pytest.approx(1024 ** 3 * 4 * 2 / 0.130)
        flat = [s for seeds in gathered for s in seeds]
        assert len(set(flat)) == len(flat)  # no two ranks draw the same realisation


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        config, steps, warmup, cpu_sample = "c2", 1, 0, 16

    assert bench.bench_reference(A()) is None
    assert capsys.readouterr().out == ""
