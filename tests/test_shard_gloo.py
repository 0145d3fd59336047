"""Multi-process (world size 2, gloo on CPU) coverage of the sharding path: every rank
evaluates its shard of a design population, one gather returns the whole population in
order, and the max-over-ranks timing reduction.  The per-design evaluation here is the
oracle's field of each design at a few points (no GPU)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from cctpy_gb300.shard import ShardedEvaluator, gather_rows, max_over_ranks, shard_by_cost, shard_range  # noqa: E402


def test_shard_range_covers_everything_once():
    for n in (0, 1, 5, 64, 65):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, world, r) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1


def test_shard_by_cost_balances():
    costs = [266400, 624960, 400000, 300000, 500000, 350000, 610000, 280000]
    world = 2
    parts = [shard_by_cost(costs, world, r) for r in range(world)]
    assert parts[0][0] == 0 and parts[-1][1] == len(costs) and parts[0][1] == parts[1][0]
    loads = [sum(costs[a:b]) for a, b in parts]
    assert max(loads) - min(loads) <= max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _design_fields(rows):
    """Oracle field of a small CCT whose current is the row's parameter, at 3 points."""
    from oracle import cct_oracle as O
    out = []
    for r in rows:
        rec = O.cct_record(O.Frame((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.0, 1.0)), 0.95, 0.083, 22.5,
                           [30.0, 80.0, 90.0, 90.0], 4, float(r[0]), (0.0, 0.0),
                           (2 * np.pi * 4, -np.deg2rad(22.5)), 36)
        m = O.CCTOracle(rec)
        out.append(np.concatenate([m.field_at(p) for p in ((0.95, 0.01, 0.0), (0.9, 0.2, 0.01), (0.8, 0.3, -0.01))]))
    return np.array(out)


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        params = np.array([[1000.0 * (k + 1)] for k in range(5)])        # 5 designs: ragged split 3 + 2
        ev = ShardedEvaluator(_design_fields, cost=lambda r: abs(r[0]))
        res = ev(params)
        empty = gather_rows(np.zeros((0,)) if rank == 1 else np.ones((2, 3)))
        t = max_over_ranks(0.5 + rank)
        q.put((rank, res, empty, t))
    finally:
        dist.destroy_process_group()


def test_sharded_population_two_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = _design_fields(np.array([[1000.0 * (k + 1)] for k in range(5)]))
    for rank, res, empty, t in got:
        np.testing.assert_array_equal(res, want)
        assert empty.shape == (2, 3) and np.all(empty == 1)
        assert t == 1.5


def _failing_eval(rows):
    raise ValueError("design evaluation failed")


def _worker_fail(rank, world, port, q):
    import datetime
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    try:
        ev = ShardedEvaluator(_failing_eval if rank == 1 else _design_fields)
        ev(np.array([[1000.0], [2000.0]]))
        q.put((rank, "returned"))
    except ValueError:          # the failing rank's own error
        q.put((rank, "ValueError"))
    except RuntimeError:        # the survivor's failed gather (torch's distributed errors derive from it)
        q.put((rank, "RuntimeError"))
    finally:
        dist.destroy_process_group()


def test_a_failing_rank_ends_the_gather_with_an_error():
    """A rank whose evaluation raises leaves the gather; the other rank's gather then fails
    (gloo: the peer closed its connection; otherwise the process group's 10 s timeout) instead
    of waiting for ever."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker_fail, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
    assert got[1] == "ValueError"
    assert got[0] == "RuntimeError"
