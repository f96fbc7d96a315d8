"""Worker of the root-sharding tests: one gloo rank of a sharded forest whose
per-rank forests are oracle stand-ins (no GPU in these tests)."""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)


class OracleForest:
    """DeviceForest-shaped wrapper of the oracle port (test stand-in)."""

    def __init__(self, g, roots):
        from oracle import oracle as orc
        self.o = orc.PortOracle(g.nv, g.off, g.adj, roots, nthreads=1)
        self.o.static()

    def insert(self, pairs):
        for u, v in np.asarray(pairs).reshape(-1, 2):
            self.o.insert(int(u), int(v))

    def delete(self, pairs):
        for u, v in np.asarray(pairs).reshape(-1, 2):
            self.o.delete(int(u), int(v))

    def bc(self):
        return self.o.bc()

    def level64(self):
        return self.o.level()

    def sigma(self):
        return self.o.sigma()


def case(name):
    from streamingbc_gb300 import graphs as G
    if name == "rmat":
        g = G.rmat(9, 8, seed=21)
        return g, G.pick_roots(g.nv, 37, seed=21), G.rmat_insertions(g, 9, 48, seed=21)
    g = G.er(300, 1200, seed=22)
    return g, G.pick_roots(g.nv, 300, seed=22), G.uniform_insertions(g, 40, seed=22)


def deletions(name):
    """Edges of the original graph removed after the insertions."""
    from streamingbc_gb300 import graphs as G
    g, _, _ = case(name)
    E = G.edge_list(g)
    return E[np.random.default_rng(23).choice(len(E), 12, replace=False)]


def run(rank, world, port, name, out_dir, fail_rank=-1):
    import torch.distributed as dist
    from streamingbc_gb300.sharding import ShardedForest
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g, roots, ins = case(name)
        sf = ShardedForest(roots, rank, world, lambda r: OracleForest(g, r))
        for s in range(0, len(ins), 16):
            sf.insert(ins[s:s + 16])
        sf.delete(deletions(name))
        bc = sf.bc()
        lv = sf.level64()
        sg = sf.sigma()
        if rank == 0:
            np.savez(os.path.join(out_dir, f"{name}_{world}.npz"), bc=bc, lv=lv, sg=sg,
                     mine=np.asarray(sf.roots))
    finally:
        dist.destroy_process_group()
