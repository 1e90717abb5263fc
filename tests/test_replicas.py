"""Multi-GPU runs of the bench are independent replicas (one graph per GPU, no data-path
collective); the only cross-rank step is taking the slowest rank's time.  These tests run
that host logic as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, w)   # per-rank step times, ms
        q.put((r, w, local, slowest))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_time_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 0, 15.0), (1, 2, 1, 15.0)]


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    """under torchrun only rank 0 runs and prints the reference line"""
    import bench
    from bruno_gb300 import synth
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        cpu_sample, warmup, steps, gpus = 0.01, 1, 1, 2
    bench.run_reference(Args(), synth.WORKLOADS["plain-small"])
    assert capsys.readouterr().out == ""


def test_reference_arm_line(monkeypatch, capsys):
    """rank 0 prints one reference line on the arm's own config: the oracle's rate over its six
    path phases, the same figure as its cpu_baseline and its e2e (no device copies)"""
    import json
    import bench
    from bruno_gb300 import synth
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    w = synth.WORKLOADS["plain-small"]

    class Args:
        ref_sample, warmup, steps, gpus = 0.5, 0, 1, 1
    bench.run_reference(Args(), w)
    lines = capsys.readouterr().out.strip().splitlines()
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["config"] == bench.workload_config(w)
    assert line["data"] == "synthetic (seeded generator, plain-small)"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] == "port" and cb["cores"] >= 1
    assert set(cb["phases_s"]) == {"parse", "count_k2mers", "filter_insert", "chainmap", "list_rank", "compress"}
    # the step time is the six phases' sum (they are rounded to 0.1 ms in the line)
    assert abs(line["ms_per_step"] - 1e3 * sum(cb["phases_s"].values())) < 1.0
    assert "first 50000 of 100000 reads (50%)" in cb["sample"]
