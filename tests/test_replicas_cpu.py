"""The multi-GPU form of the benchmark is replicas only (the path has no
data-path exchange): every rank runs its own dgesv, the job's time is the
slowest rank's (a max all-reduce) and the throughput is the ranks' work over
that time.  This checks that host logic with two `gloo` ranks on the CPU,
and that the reference arm leaves all work to rank 0."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    own_ms = [120.0, 150.0][rank]                      # rank 1 is the slow one
    job_ms = bench.max_over_ranks(dist, own_ms, "cpu")
    value = bench.replica_throughput(world, 3.0e11, 4, job_ms)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"job_ms": job_ms, "value": value}, f)


def test_two_gloo_ranks_take_the_slowest_rank(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for g in got:
        assert g["job_ms"] == 150.0
        assert g["value"] == pytest.approx(2 * 3.0e11 * 4 / 0.150 / 1e12)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 42.5, "cpu") == 42.5
    assert bench.replica_throughput(1, 1e12, 2, 1000.0) == pytest.approx(2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup, gpus = 1, 0, 2
    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
