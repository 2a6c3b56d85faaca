"""Multi-GPU form (replicas) on the CPU: two gloo ranks.

Every rank solves its own batch; the only collective work is host
bookkeeping -- a barrier, the slowest rank's time, one reporting rank -- and
throughput is all ranks' units over that time.  The reference arm of the
bench runs on rank 0 alone.
"""
import argparse
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from geopvi_gb300.replicas import ReplicaGroup
    g = ReplicaGroup(backend="gloo")
    g.barrier()
    slowest = g.max_seconds(0.1 * (rank + 1))      # rank r took 0.1 (r + 1) s
    rate = g.throughput(1000.0, slowest)            # 1000 units per rank
    q.put((g.rank, g.world, g.reporter, slowest, rate))
    g.close()


@pytest.mark.parametrize("world", [2, 3])
def test_replica_bookkeeping_over_gloo(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 0.1 * world
    for rank, w, reporter, m, rate in results:
        assert w == world and reporter == (rank == 0)
        assert m == pytest.approx(slowest)
        assert rate == pytest.approx(1000.0 * world / slowest)


def test_single_process_needs_no_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from geopvi_gb300.replicas import ReplicaGroup
    g = ReplicaGroup()
    assert (g.world, g.rank, g.reporter) == (1, 0, True)
    g.barrier()
    assert g.max_seconds(0.25) == 0.25 and g.throughput(10.0, 0.5) == 20.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(config="cfg2", nt=None, cpu_shots=1, warmup=0, steps=1)
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
