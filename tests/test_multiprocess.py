"""The multi-GPU path is replicas only: each rank reconstructs its own batch,
and the ranks meet only for the timing barrier and the max of their step
times (gloo, host side).  These tests run that path as two CPU processes
with the gloo backend on 127.0.0.1, and check the reference arm's rank
rule (rank 0 alone runs and prints)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, values, out):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench

    r, w, local, pg = bench.dist_init(world)
    assert (r, w, local) == (rank, world, rank) and pg is not None
    bench.barrier(pg)
    got = bench.allmax(pg, values[rank])
    bench.barrier(pg)
    pg.destroy_process_group()
    out.put((rank, got))


@pytest.mark.parametrize("values", [(3.5, 1.25), (0.5, 7.0)])
def test_two_ranks_barrier_and_max_over_ranks(values):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank times the step as the slowest rank's time
    assert res == {0: max(values), 1: max(values)}


def test_single_process_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    rank, world, local, pg = bench.dist_init(1)
    assert (rank, world, local, pg) == (0, 1, 0, None)
    bench.barrier(pg)
    assert bench.allmax(pg, 2.5) == 2.5


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    # ranks other than 0 return at once, without work or output
    assert bench.reference_arm(None, {}, 1, 2, None) == 0
    assert capsys.readouterr().out == ""
