"""Root sharding across processes (one GPU each).

Trees of different roots are independent (the reference's COARSE loop runs
them in parallel, src/streamingbc.c:171-208), so a forest of K roots splits
across ranks by roots: rank r owns roots[r::world] with their dist/sigma/delta.
The graph is replicated: every rank appends every insertion, in the same
order, to its own copy of the adjacency.  Each rank's BC vector is the sum of
its own roots' dependencies, so the only exchange step is one reduce-sum of
the partial BC vectors, done when BC is read -- nothing is exchanged per
insertion.

The forest behind each rank is anything with the DeviceForest methods used
here (insert, bc, level64, sigma), so the same logic runs over GPU forests in
production and over CPU stand-ins in the multi-process tests.
"""
from __future__ import annotations

import numpy as np


def shard_roots(roots, rank: int, world: int) -> np.ndarray:
    """Roots owned by `rank`: every world-th root starting at rank (strided,
    so ranks get statistically equal shares of a uniformly drawn root set)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    return np.ascontiguousarray(np.asarray(roots, dtype=np.int64)[rank::world])


def reduce_sum(x: np.ndarray, group=None) -> np.ndarray:
    """All-reduce sum of a float64 vector over the process group (gloo on CPU
    tensors, NCCL on CUDA tensors)."""
    import torch
    import torch.distributed as dist
    backend = dist.get_backend(group)
    t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64))
    if backend == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def gather_rows(rows: np.ndarray, world: int, group=None) -> np.ndarray:
    """Re-assemble per-root rows of a strided shard on every rank: rank r's
    row j is global root r + j*world.  Used to compare a sharded forest's
    full state with an unsharded one."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(rows))
    n = torch.tensor([t.shape[0]], dtype=torch.int64)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    cap = int(max(s.item() for s in sizes))
    pad = torch.zeros((cap,) + tuple(t.shape[1:]), dtype=t.dtype)
    pad[: t.shape[0]] = t
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    total = int(sum(s.item() for s in sizes))
    out = np.zeros((total,) + tuple(t.shape[1:]), dtype=rows.dtype)
    for r in range(world):
        k = int(sizes[r].item())
        out[r::world][:k] = parts[r][:k].numpy()
    return out


class ShardedForest:
    """One rank's share of a root-sharded forest.

    make_forest(roots) builds this rank's forest over its own copy of the
    graph and runs the static init; insertions and deletions go to every rank
    in the same order; bc() reduces the partial BC vectors over the group."""

    def __init__(self, roots, rank: int, world: int, make_forest, group=None):
        self.rank, self.world, self.group = rank, world, group
        self.all_roots = np.asarray(roots, dtype=np.int64)
        self.roots = shard_roots(self.all_roots, rank, world)
        self.forest = make_forest(self.roots)

    def insert(self, pairs):
        """Apply a batch of insertions (the same batch on every rank)."""
        return self.forest.insert(pairs)

    def delete(self, pairs):
        """Apply a batch of edge deletions, in order (the same batch on every
        rank; each rank's graph copy loses the edges, its roots are updated)."""
        return self.forest.delete(pairs)

    def partial_bc(self) -> np.ndarray:
        return np.asarray(self.forest.bc(), dtype=np.float64)

    def bc(self) -> np.ndarray:
        """BC over all roots of all ranks (collective: every rank calls it)."""
        if self.world == 1:
            return self.partial_bc()
        return reduce_sum(self.partial_bc(), self.group)

    def level64(self) -> np.ndarray:
        """Full [K][V] levels (collective)."""
        mine = np.asarray(self.forest.level64())
        return mine if self.world == 1 else gather_rows(mine, self.world, self.group)

    def sigma(self) -> np.ndarray:
        mine = np.asarray(self.forest.sigma())
        return mine if self.world == 1 else gather_rows(mine, self.world, self.group)
