"""Generate the golden vectors in this folder from the UNMODIFIED reference.

Runs the reference's COARSE path (compiled from its own sources by
``make -C oracle ref`` into oracle/_ref/libsbcref.so, driven by
oracle/ref_harness.c) on small graphs and records its outputs:
static-init level/sigma/BC, the BC vector after every insertion, the final
level/sigma/BC and the reference's traversal counters per insertion.

Cases:
  karate, dolphins   the reference's bundled DIMACS graphs (graphs/*.graph),
                     0-based ids without the DIMACS dummy vertex, exact BC.
  er200              ER G(200, 600) seed 21, 64 sampled roots.
  er200sparse        ER G(200, 150) seed 22 (many components), exact BC;
                     insertions join components (|d| > 1 from "infinity").
  rmat9              R-MAT scale 9, edge factor 8, seed 23, 64 roots,
                     R-MAT-drawn insertions (isolated vertices present).

Usage (only where the reference tree and a C compiler exist):
    python tests/golden/make_golden.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from streamingbc_gb300 import graphs as G  # noqa: E402


def read_dimacs(path: str) -> G.Graph:
    with open(path) as fh:
        head = fh.readline().split()
        n = int(head[0])
        us, vs = [], []
        for u in range(n):
            line = fh.readline()
            for tok in line.split():
                us.append(u)
                vs.append(int(tok) - 1)
    return G.from_edges(n, np.array(us), np.array(vs))


def run_case(name, g, roots, ins):
    r = orc.RefOracle(g.nv, g.off, g.adj, roots, nthreads=1)
    r.static()
    lv0, sg0, _, bc0 = r.dump()
    trace = np.zeros((len(ins), g.nv))
    counters = np.zeros((len(ins), 4), dtype=np.int64)
    for i, (u, v) in enumerate(ins):
        r.insert(int(u), int(v))
        c = r.counters()
        counters[i] = [c["vertices"], c["edges"], c["case1"], c["case2"]]
        trace[i] = r.dump()[3]
    lv1, sg1, _, bc1 = r.dump()
    r.close()
    out = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(out, nv=g.nv, off=g.off, adj=g.adj, roots=roots, ins=ins,
                        level0=lv0, sigma0=sg0, bc0=bc0, level1=lv1, sigma1=sg1, bc1=bc1,
                        bc_trace=trace, counters=counters)
    print(name, g.nv, g.ne, len(roots), len(ins), os.path.getsize(out))


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    orc.build(ref=True)
    for nm in ("karate", "dolphins"):
        g = read_dimacs(os.path.join(ref_root, "graphs", f"{nm}.graph"))
        run_case(nm, g, G.pick_roots(g.nv, g.nv, 0), G.uniform_insertions(g, 24, seed=11))
    g = G.er(200, 600, seed=21)
    run_case("er200", g, G.pick_roots(g.nv, 64, seed=21), G.uniform_insertions(g, 48, seed=21))
    g = G.er(200, 150, seed=22)
    run_case("er200sparse", g, G.pick_roots(g.nv, g.nv, 0), G.uniform_insertions(g, 48, seed=22))
    g = G.rmat(9, 8, seed=23)
    run_case("rmat9", g, G.pick_roots(g.nv, 64, seed=23), G.rmat_insertions(g, 9, 48, seed=23))


if __name__ == "__main__":
    main()
