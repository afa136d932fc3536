"""Multi-rank logic of bench.py on CPU: two gloo ranks on 127.0.0.1.

The bench runs one replica of the iteration per GPU; the job's time is the
slowest rank's and its rate counts every rank's steps.  The reference arm runs
on rank 0 alone.
"""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r timed 10 (r + 1) ms for 5 steps
        ms, rate = bench.job_rate(10.0 * (rank + 1), 5, world, "cpu")
        alone = bench.max_over_ranks(3.0 + rank, world, "cpu")
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{ms!r} {rate!r} {alone!r}\n")
    finally:
        dist.destroy_process_group()


def test_job_rate_takes_the_slowest_rank(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for r in range(world):
        ms, rate, alone = (float(x) for x in open(tmp_path / f"rank{r}.txt").read().split())
        assert ms == 20.0  # every rank sees the slowest rank's time
        assert rate == pytest.approx(world * 5 / 0.020)  # 10 steps over 20 ms
        assert alone == 4.0


def test_job_rate_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    ms, rate = bench.job_rate(8.0, 4, 1, "cpu")
    assert ms == 8.0 and rate == pytest.approx(500.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Ranks other than 0 exit without work (nothing built, nothing printed)."""
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "build_workload", lambda: called.append(1))
    bench.run_reference(type("A", (), {"warmup": 3, "steps": 2})())
    assert not called
    assert capsys.readouterr().out == ""
