"""The N > 1 host path (independent replicas, max-over-ranks timing, rank-0
reporting) on two CPU ranks with gloo."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from mbsymmetry_gb300.replicas import Replicas
    r = Replicas("gloo")
    r.barrier()
    ms = 10.0 + 5.0 * rank                     # each replica's own time
    ms_max = r.max_over_ranks(ms)
    q.put((rank, ms_max, r.seconds_per_iteration(ms_max), r.replica_throughput(ms_max), r.reports))
    r.close()


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(world))
    assert [o[1] for o in out] == [15.0, 15.0]                 # both ranks see the slowest replica
    assert [o[2] for o in out] == [15.0 / 1e3] * 2             # one iteration takes the slowest time
    assert [o[3] for o in out] == [2 / 15e-3] * 2              # two independent iterations in it
    assert [o[4] for o in out] == [True, False]                # rank 0 reports


def test_single_process_defaults(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from mbsymmetry_gb300.replicas import Replicas
    r = Replicas()
    assert (r.rank, r.world) == (0, 1) and r.reports
    assert r.max_over_ranks(3.5) == 3.5 and r.seconds_per_iteration(100.0) == 0.1
    assert r.replica_throughput(100.0) == 10.0
