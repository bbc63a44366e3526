"""The N > 1 path of bench.py on CPU: two replica ranks over gloo (127.0.0.1).

The benchmark runs one independent factorization per GPU (replicas, no
collective on the data path): the job's step time is the slowest rank's
(max over ranks), and the whole-job throughput is every rank's work over that
time. These tests run the same helpers the benchmark uses with the gloo
backend and CPU tensors, and check that the reference arm's other ranks exit
without work."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, step_s, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist = bench.dist_setup(None, backend="gloo")
    try:
        dist.barrier()
        t = bench.max_over_ranks(dist, step_s[rank], device="cpu")
        v = bench.replica_throughput(100.0, w, t)
        dist.barrier()
        q.put((r, w, local, t, v))
    finally:
        dist.destroy_process_group()


def _run(world, step_s):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, step_s, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_two_replicas_take_the_slowest_rank_time():
    out = _run(2, [0.5, 0.75])
    for r, (rank, world, local, t, v) in enumerate(out):
        assert (rank, world, local) == (r, 2, r)
        assert t == 0.75                      # every rank sees the slowest replica
        assert v == pytest.approx(100.0 * 2 / 0.75)  # both ranks' work over that time


def test_single_process_needs_no_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    world, rank, local, dist = bench.dist_setup(None)
    assert (world, rank, local, dist) == (1, 0, 0, None)
    assert bench.max_over_ranks(None, 0.3) == 0.3
    assert bench.replica_throughput(10.0, 1, 0.5) == 20.0


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        n, nrhs, steps, warmup, ref_step_seconds = 64, 1, 1, 3, 0.01

    assert bench.run_reference(Args()) is None
    assert capsys.readouterr().out == ""


def test_reference_arm_rank0_prints_one_line(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "0")
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        n, nrhs, steps, warmup, ref_step_seconds, arith = 96, 1, 1, 3, 0.01, "fast"

    bench.run_reference(Args())
    lines = [l for l in capsys.readouterr().out.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    # the same workload description as the library's own line
    assert d["config"] == bench.bench_config(Args(), bench.DEFAULT_PANEL_WIDTH, 2)
