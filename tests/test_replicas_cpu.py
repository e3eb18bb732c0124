"""The multi-GPU form of the benchmark is independent replicas (one cube per rank, no data-path collective): its host
logic, run as two gloo ranks on the CPU — the max-over-ranks step time, the whole-job rate, and the reference arm
printing from rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_info()
    assert (r, w, local) == (rank, world, rank)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, w, torch.device("cpu"))   # rank 1 is the slow replica
    rate = bench.job_rate(1000, w, ms / 1e3)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, rate))


@pytest.mark.timeout(120)
def test_two_gloo_replicas_time_by_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=100) for _ in range(world))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for rank, ms, rate in got:
        assert ms == 15.0                     # every rank sees the slowest replica's time
        assert rate == pytest.approx(2 * 1000 / 0.015)


def test_reference_arm_prints_on_rank_zero_only(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 1, 0, 2
    bench.run_reference(A())                  # returns before any work on ranks other than 0
    assert capsys.readouterr().out == ""
