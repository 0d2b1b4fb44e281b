"""Replica harness of bench.py on CPU: two gloo ranks.  The single scene is
not sharded; each rank runs an independent replica and the job's time is the
slowest rank's.  This checks the max-over-ranks reduction, the timed
replica loop bench.py's headline runs (barrier, steps between the timer's
marks, slowest rank, aggregate of every rank's work) driven with a fake
step, and that the reference arm only works on rank 0."""
from __future__ import annotations

import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_info()
        t_local = 1.0 + rank  # rank 1 is the slow one
        t = bench.reduce_max(dist, t_local)
        n, steps = 1000, 10
        value = w * n * bench.ITERATIONS * steps / t
        dist.barrier()
        q.put((rank, w, r, t, value))
    finally:
        dist.destroy_process_group()


class _FakeReplica:
    """Stands in for a Simulation: a step takes a fixed host time."""

    def __init__(self, step_s: float):
        self.step_s = step_s
        self.steps = 0
        self.syncs = 0

    def step(self, n: int, sync: bool = True):
        import time

        time.sleep(self.step_s * n)
        self.steps += n

    def sync(self):
        self.syncs += 1


def _replica_worker(rank: int, world: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sim = _FakeReplica(0.02 * (rank + 1))  # rank 1 steps twice as slowly
        before = []
        t, value = bench.timed_replica_steps(dist, sim, 5, bench.WallTimer(), 1000,
                                             before=lambda: before.append(1))
        q.put((rank, t, value, sim.steps, sim.syncs, len(before)))
    finally:
        dist.destroy_process_group()


def test_timed_replica_steps_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + ((os.getpid() + 500) % 1000)
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    times = {t for _, t, *_ in out}
    assert len(times) == 1  # every rank reports the slowest rank's time
    t = times.pop()
    assert 0.2 <= t < 0.6  # rank 1: 5 steps x 40 ms
    for rank, _, value, steps, syncs, before in out:
        assert steps == 5 and syncs == 2 and before == 1
        assert value == pytest.approx(2 * 1000 * 4 * 5 / t)


def test_two_gloo_ranks_reduce_to_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, w, r, t, value in out:
        assert w == 2 and r == rank
        assert t == 2.0
        assert value == pytest.approx(2 * 1000 * 4 * 10 / 2.0)


def test_reference_arm_is_rank0_only(monkeypatch, capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup, gpus, cpu_budget, workload = 1, 3, 2, 0.1, "single"

    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
