"""Multi-rank host logic of the benchmark on CPU (gloo, world size 2): the
replicas' slowest time is agreed by every rank and the whole-job rate counts
every replica's work; the reference arm runs on rank 0 only."""
import os
import socket
import sys
import tempfile

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _entry(rank, world, port, out_dir):
    sys.path.insert(0, HERE)
    import multirank_worker
    multirank_worker.run(rank, world, port, out_dir)


def test_max_over_ranks_and_rate_gloo():
    work = os.path.join(ROOT, "pycbf_gb300", "_build")
    os.makedirs(work, exist_ok=True)
    with tempfile.TemporaryDirectory(dir=work) as d:
        mp.start_processes(_entry, args=(2, _free_port(), d), nprocs=2, join=True,
                           start_method="spawn")
        for rank in range(2):
            with open(os.path.join(d, f"rank{rank}.txt")) as fp:
                slowest, rate = map(float, fp.read().split())
            assert slowest == 2.5
            assert rate == pytest.approx(2 * 1000.0 / 2.5)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, "cpu") == 3.25
    assert bench.replicas_rate(1, 10.0, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference_arm(None) is None
    assert capsys.readouterr().out == ""
