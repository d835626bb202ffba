"""The N > 1 host logic of bench.py on two CPU ranks over gloo: one rendezvous on 127.0.0.1,
the max-over-ranks timing every rank agrees on, the barrier, each rank's own shard of independent
batch problems of one seeded batch, bin-packed by per-step work (no data-path collective; the
final states are gathered on rank 0), and the reference arm running on rank 0 only.  The
single-problem step does not shard (replicas); the batch does."""
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
        import numpy as np
        from pyprop_gb300.batch import gather_states, random_batch, shard as shard_of, step_bytes
        # one seeded batch, this rank's bin-packed share of it, a per-problem result gathered on rank 0
        full = random_batch(12, seed=20261204, lmax=(2, 9), nr=(30, 90), rmax=(20.0, 60.0))
        plan = shard_of(full, w)
        mine = plan[r]
        states = [full[i].initial_state() for i in mine]
        got = gather_states(states, mine, w, len(full))
        ok = None
        if r == 0:
            ok = all(np.array_equal(got[i], full[i].initial_state()) for i in range(len(full)))
        loads = [sum(step_bytes(full[i]) for i in part) for part in plan]
        shard = (mine, plan, loads, ok)
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
    (mine0, plan0, loads, ok), (mine1, plan1, _, ok1) = res[0][3], res[1][3]
    assert plan0 == plan1                                  # every rank computes the same plan
    assert sorted(mine0 + mine1) == list(range(12)) and not set(mine0) & set(mine1)   # disjoint, complete
    assert max(loads) <= 1.05 * (sum(loads) / 2)           # per-step work balanced within 5%
    assert ok is True and ok1 is None                      # rank 0 holds every problem's state
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
