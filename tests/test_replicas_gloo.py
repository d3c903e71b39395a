"""Multi-rank host logic of bench.py on CPU (gloo, 2 ranks): the path runs as
independent replicas, one per GPU, with no collective in the data path; the
only cross-rank steps are the barrier and the max over ranks of the timed
region, from which the whole-job rate is formed.  Under torchrun the reference
arm runs on rank 0 alone and the other ranks exit without work."""
import importlib.util
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        b = _bench()
        local_ms = 10.0 + 5.0 * rank          # rank 1 is the slower replica
        slowest = b.max_over_ranks(local_ms, "cpu")
        rate = b.job_rate(world, 7, slowest / 1e3)
        dist.barrier()
        q.put((rank, slowest, rate))
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in out] == [0, 1]
    for _, slowest, rate in out:
        assert slowest == 15.0                  # every rank sees the max
        assert rate == pytest.approx(2 * 7 / 0.015)


def test_single_process_needs_no_group():
    b = _bench()
    assert b.max_over_ranks(3.5) == 3.5
    assert b.job_rate(1, 4, 2.0) == 2.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    b = _bench()
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3"])
    b.main()                                    # returns at once: no work, no output, no device
    assert capsys.readouterr().out == ""
