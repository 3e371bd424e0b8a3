"""Host logic of bench.py's multi-rank run (replicas, barrier, max over ranks) on gloo, world_size 2."""

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "CUDA_VISIBLE_DEVICES": ""})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r, _ = bench._dist()
    bench._barrier(w)
    # rank r "took" 1 + r seconds for 10 steps: the job's time is the slowest rank's
    value, total = bench._aggregate(w, 10, 1.0 + r)
    q.put((r, w, value, total))
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, value, total) in enumerate(out):
        assert (rank, world) == (r, 2)
        assert total == pytest.approx(2.0)          # max over ranks
        assert value == pytest.approx(2 * 10 / 2.0)  # all ranks' units / slowest time


def test_single_rank_aggregate_is_local():
    sys.path.insert(0, ROOT)
    import bench

    assert bench._aggregate(1, 30, 1.5) == (20.0, 1.5)


def test_reference_arm_nonzero_rank_does_no_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_reference", lambda *a, **k: called.append(1))

    class A:
        steps, cpu_budget, small, gpus = 3, 1.0, True, 2

    bench.run_reference(A())
    assert not called and capsys.readouterr().out == ""


def test_reference_arm_prints_the_gpu_arms_config(monkeypatch, capsys):
    """The reference arm's line names the same workload configuration as the
    GPU arm's (headline_config), so that the two lines compare like for like."""
    sys.path.insert(0, ROOT)
    import json

    import bench

    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setattr(bench, "cpu_reference", lambda *a, **k: {
        "value": 30.0, "unit": "iter/s", "cores": 16, "kind": "port", "sample": "stub", "iters": 3, "warmup": 1})

    class A:
        steps, warmup, cpu_budget, small, gpus = 3, 1, 1.0, False, 1

    bench.run_reference(A())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["config"] == bench.headline_config(False, 1)
    assert line["config"]["n_tets"] == 1_500_000 and line["config"]["n_vertices"] == 314_721
    assert line["metric"] == bench.METRIC and line["unit"] == "iter/s" and line["higher_is_better"]
