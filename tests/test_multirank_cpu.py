"""The N > 1 host logic of bench.py on two CPU ranks over gloo: one rendezvous on 127.0.0.1,
the max-over-ranks timing every rank agrees on, the barrier, each rank's own shard of independent
batch problems (no data-path collective), and the reference arm running on rank 0 only.  The
single-problem step does not shard (replicas); the batch does (weak scaling)."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                          WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
        sys.path.insert(0, ROOT)
        import torch.distributed as dist
        dist.init_process_group("gloo", rank=rank, world_size=world)
        import bench
        r, w, _ = bench._dist()
        t = bench._max_over_ranks(1.5 * (r + 1), w)          # per-rank "elapsed" seconds
        bench._barrier(w)
        from pyprop_gb300.batch import random_batch
        shard = [(p.lmax, p.nr, p.m, round(p.rmax, 6)) for p in random_batch(4, seed=20261204 + r)]
        # the reference arm: rank 0 does the work, every other rank returns at once, silent
        out = io.StringIO()
        if r != 0:
            with redirect_stdout(out):
                bench.run_reference(None, r, w)
        dist.destroy_process_group()
        q.put((r, w, t, shard, out.getvalue()))
    except Exception as e:  # surfaced by the parent
        q.put((rank, -1, repr(e), None, ""))


def test_two_rank_timing_barrier_and_batch_shards():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=300) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
    for r, w, t, shard, out in res:
        assert w == 2, t
    assert [x[2] for x in res] == [3.0, 3.0]              # max over ranks, seen by both
    assert res[0][3] != res[1][3]                          # each rank its own shard of problems
    assert res[1][4] == ""                                 # no reference work or output on rank 1
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_helpers_need_no_process_group(monkeypatch):
    """At N = 1 the helpers are plain pass-throughs (no torch.distributed initialisation)."""
    sys.path.insert(0, ROOT)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert bench._dist() == (0, 1, 0)
    assert bench._max_over_ranks(2.5, 1) == 2.5
    bench._barrier(1)
