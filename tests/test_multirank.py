"""bench.py's multi-rank host logic on CPU: two `gloo` ranks on 127.0.0.1.

`bench.py --gpus N` runs N replicas of the transfer, one rank per GPU, with no
data-path collective; the job's step time is the slowest rank's (an all-reduce
MAX of the timed totals, for the kernel-timed value and for e2e), and the
job's value is N x the particles per rank over that time. The reference arm
runs on rank 0 alone; the other ranks exit 0 without output.
"""
import os
import socket

import pytest

import bench


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", rank=rank, world_size=world)
        r, w, local = bench.dist_info()
        # rank r took 10 + 5 r ms: every rank must see the slowest one
        t = bench.max_over_ranks(10.0 + 5.0 * r, w, "cpu")
        dist.barrier()
        q.put((r, w, local, t, bench.job_value(1000, w, t)))
        dist.destroy_process_group()
    except Exception as e:  # reported to the parent, which fails the test
        q.put(("error", rank, repr(e)))


def test_two_ranks_use_the_slowest_rank_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    world = 2
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        results = [q.get(timeout=120) for _ in range(world)]
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
    errors = [r for r in results if r[0] == "error"]
    assert not errors, errors
    assert sorted(r[0] for r in results) == [0, 1]
    for r, w, local, t, value in results:
        assert w == 2 and local == r
        assert t == 15.0
        # 2 ranks x 1000 particles in 15 ms
        assert value == pytest.approx(2000 / 0.015)
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(7.5, 1, "cpu") == 7.5
    assert bench.job_value(1 << 27, 1, 14.28) == pytest.approx((1 << 27) / 0.01428)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(None) == 0
    assert capsys.readouterr().out == ""
