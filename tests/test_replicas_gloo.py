"""Multi-rank host logic of the benchmark (replicas only), on CPU with two gloo
ranks: the timed region is the maximum over ranks, the value the aggregate of
the replicas, every rank starts its own seeded system, and the reference arm
runs on rank 0 alone."""
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


def _rank(rank, world, port, times, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, v = bench.replica_timing(times[rank], 100, world, dist, "cpu")
    out.put((rank, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_max_time_and_the_aggregate_value():
    sys.path.insert(0, ROOT)
    import bench

    world, times = 2, [0.040, 0.055]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, times, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == pytest.approx(0.055)
        assert v == pytest.approx(2 * bench.ns_per_day(0.055 / 100))


def test_single_rank_keeps_its_own_time():
    sys.path.insert(0, ROOT)
    import bench

    t, v = bench.replica_timing(0.03, 10, 1)
    assert t == 0.03 and v == pytest.approx(bench.ns_per_day(0.003))


def test_replica_starts_differ_by_rank():
    from qtip4pf_water_gb300.start import seeded_start

    import numpy as np

    a = seeded_start(8, 2, 298.0, seed=2024)
    b = seeded_start(8, 2, 298.0, seed=2025)
    assert not np.array_equal(a.q, b.q)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    bench.run_reference(argparse.Namespace(steps=1, warmup=3, gpus=2, impl="reference", cpu_seconds=1.0))
    assert capsys.readouterr().out == ""
