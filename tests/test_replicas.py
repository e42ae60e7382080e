"""The multi-GPU layout is replicas only (independent films, no collective on
the data path): bench.py's N > 1 bookkeeping -- the slowest rank's time and
the whole-job rate -- checked with two gloo ranks on the CPU, and the
reference arm's rank > 0 exit without work."""
import os
import socket

import pytest

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank
        q.put((rank, bench.max_over_ranks(ms, dist, "cpu")))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 15.0, 1: 15.0}


def test_single_rank_and_rate():
    assert bench.max_over_ranks(7.5) == 7.5
    # two replicas of 2^21 cells, 20 steps in 4 ms: 2 * 2^21 * 20 / 4e-3
    assert bench.replica_rate(1 << 21, 20, 4.0, 2) == pytest.approx(2 * (1 << 21) * 20 / 4e-3)


def test_reference_arm_other_ranks_exit(monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.dist_env() == (2, 1, 0)
    assert bench.run_reference(None) == 0
