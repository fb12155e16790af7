"""bench.py under torchrun: every rank advects its own copy of the workload
(the path is not sharded), and the reported value is the units of all ranks
over the slowest rank's time.  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, w, dist = bench.dist_setup()
    try:
        bench.dist_barrier(dist)
        # rank r processed (r + 1) * 1000 units in (r + 1) * 0.5 s
        units, secs = bench.replica_totals((r + 1) * 1000, (r + 1) * 0.5, dist)
        q.put((r, w, dist.get_backend(), units, secs))
    finally:
        dist.destroy_process_group()


def test_replica_totals_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the CPU form of this test runs where no GPU is visible (gloo backend)")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=5) for _ in range(2))
    for r, (rank, world, backend, units, secs) in enumerate(got):
        assert (rank, world, backend) == (r, 2, "gloo")
        assert units == 3000.0  # sum over ranks
        assert secs == 1.0      # slowest rank


def test_single_process_needs_no_process_group(monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    import bench
    assert bench.dist_setup() == (0, 1, None)
    assert bench.replica_totals(12, 3.0, None) == (12.0, 3.0)
