"""Multi-GPU sharding of the tracking path: one process per GPU, designs (and particle blocks)
split across ranks, no collective inside the RK4 loop.

(design, particle) pairs are independent, so a population of designs is cut into contiguous
shards, each rank tracks and reads out its shard on its own GPU, and one host-side gather
returns the objectives (or final records) of the whole population in design order.  The
gather moves (designs x 11) doubles, nothing on the data path.  torch.distributed carries
it (NCCL on GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Callable, Optional, Sequence, Tuple

import numpy as np
import torch


def shard_range(n: int, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of n items for `rank` of `world`: the first n % world ranks
    get one item more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    if n < 0:
        raise ValueError(f"negative item count {n}")
    q, r = divmod(n, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def shard_by_cost(costs: Sequence[float], world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of items with per-item `costs` (e.g. segment counts) so that
    every rank's share of the total cost is as even as contiguous cuts allow: cut k is put
    before or after the item where the running cost crosses k / world of the total,
    whichever lands closer."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    c = np.cumsum(np.asarray(costs, dtype=np.float64))
    n = len(c)
    cuts = [0]
    for k in range(1, world):
        target = c[-1] * k / world if n else 0.0
        i = int(np.searchsorted(c, target, side="left"))
        if i >= n:
            cut = n
        else:
            before = c[i - 1] if i > 0 else 0.0
            cut = i if abs(before - target) <= abs(c[i] - target) else i + 1
        cuts.append(max(cut, cuts[-1]))
    cuts.append(n)
    return cuts[rank], cuts[rank + 1]


def gather_rows(local: np.ndarray, group=None) -> np.ndarray:
    """Concatenation, in rank order, of every rank's `local` rows ((m_rank, ...) float64, at
    most three trailing dimensions; a rank without rows may pass np.zeros((0,))): all-gather
    of the shapes, then of the rows padded to the largest count."""
    import torch.distributed as dist
    local = np.ascontiguousarray(local, dtype=np.float64)
    if local.ndim > 4:
        raise ValueError("rows with more than three trailing dimensions")
    world = dist.get_world_size(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")
    shape = [local.shape[0], local.ndim - 1] + list(local.shape[1:]) + [0] * (4 - local.ndim)
    shapes = [torch.zeros(5, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(shapes, torch.tensor(shape, dtype=torch.int64, device=dev), group=group)
    shapes = [s.cpu().tolist() for s in shapes]
    counts = [s[0] for s in shapes]
    full = [s for s in shapes if s[0] > 0]
    tail = tuple(full[0][2:2 + full[0][1]]) if full else tuple(local.shape[1:])
    if any(tuple(s[2:2 + s[1]]) != tail for s in full):
        raise ValueError(f"ranks disagree on the row shape: {shapes}")
    width = int(np.prod(tail)) if tail else 1
    m = max(counts) if counts else 0
    pad = torch.zeros((m, width), dtype=torch.float64, device=dev)
    if local.shape[0]:
        pad[:local.shape[0]] = torch.from_numpy(local.reshape(local.shape[0], width)).to(dev)
    bufs = [torch.empty((m, width), dtype=torch.float64, device=dev) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    rows = np.concatenate([b[:k].cpu().numpy() for b, k in zip(bufs, counts)], axis=0)
    return rows.reshape((sum(counts),) + tail)


def max_over_ranks(value: float, group=None) -> float:
    """The largest of every rank's `value` (a timing, so the slowest GPU sets the clock)."""
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ShardedEvaluator:
    """A population evaluator spread over the ranks of a process group: each rank applies
    `evaluate` (e.g. an optim.GenerationEvaluator on its own GPU) to its contiguous shard of
    the parameter rows (balanced by `cost(row)` when given), and every rank gets the whole
    population's results in row order."""

    def __init__(self, evaluate: Callable[[np.ndarray], np.ndarray], cost: Optional[Callable[[np.ndarray], float]] = None,
                 group=None):
        self.evaluate, self.cost, self.group = evaluate, cost, group

    def __call__(self, params) -> np.ndarray:
        import torch.distributed as dist
        params = np.atleast_2d(np.asarray(params))
        world, rank = dist.get_world_size(self.group), dist.get_rank(self.group)
        if self.cost is None:
            a, b = shard_range(params.shape[0], world, rank)
        else:
            a, b = shard_by_cost([self.cost(r) for r in params], world, rank)
        local = np.asarray(self.evaluate(params[a:b]), dtype=np.float64) if b > a else np.zeros((0,))
        return gather_rows(local, self.group)
