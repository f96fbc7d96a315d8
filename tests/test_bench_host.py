"""Host-side pieces of the benchmark and the graph helpers the parity tests
rely on (no GPU)."""
from __future__ import annotations

import json
import os

import numpy as np

import bench
from streamingbc_gb300 import graphs as G


def test_traffic_estimate_only_for_the_captured_case_and_sources(monkeypatch):
    path = os.path.join(bench.ROOT, "profiles", "k_update_traffic.json")
    cap = json.load(open(path))["captures"][0]
    cur = cap["source_hash"]
    monkeypatch.setattr(bench, "kernel_source_hash", lambda: cur)
    wl, roots, workers, batch = cap["case"].split("/")
    roots, workers, batch = int(roots.split()[0]), int(workers.split()[0]), int(batch.split()[1])
    alg = 2.0e9
    t, why = bench.traffic_estimate(wl, batch, alg, roots, workers)
    ratio = cap["dram_bytes_per_launch"] / cap["alg_bytes_per_launch"]
    assert t is not None and abs(t - ratio * alg) < 1e-6 * alg and cur in why
    # another case: no number, and the reason says so
    t, why = bench.traffic_estimate(wl, batch, alg, roots * 2, workers)
    assert t is None and "no ncu capture" in why
    # other kernel sources: no number
    monkeypatch.setattr(bench, "kernel_source_hash", lambda: "0" * 16)
    t, why = bench.traffic_estimate(wl, batch, alg, roots, workers)
    assert t is None and "other kernel sources" in why


def test_edge_list_and_delete_edges():
    g = G.er(300, 1200, seed=4)
    E = G.edge_list(g)
    assert len(E) == g.ne and np.all(E[:, 0] < E[:, 1])
    rng = np.random.default_rng(4)
    dels = E[rng.choice(len(E), 40, replace=False)]
    # either orientation, plus an absent pair, which is ignored
    mixed = np.concatenate([dels[:20], dels[20:, ::-1]])
    present = set(map(tuple, E.tolist()))
    absent = next((u, v) for u in range(300) for v in range(u + 1, 300) if (u, v) not in present)
    g2 = G.delete_edges(g, np.concatenate([mixed, [absent]]))
    E2 = set(map(tuple, G.edge_list(g2).tolist()))
    assert E2 == present - set(map(tuple, dels.tolist()))
    assert g2.nv == g.nv and np.all(np.diff(g2.off) >= 0)
