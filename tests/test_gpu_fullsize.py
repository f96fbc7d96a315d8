"""Parity at the full sizes of the benchmarked configurations.

The other GPU tests pin every code path on graphs the oracle finishes in
seconds.  These run the configurations the benchmark times, at their stated
sizes, through the same entry points and schedules the benchmark uses, and
compare with the oracle (the reference COARSE path restated in C):

* R-MAT scale 20, K = 1024 (the headline configuration): the benchmark's own
  path -- per-job cost logging over the first 16,384 insertions, cost-model
  training, the model schedule, the launch-shape tuner, then captured device
  batches of 256, then one call of 32 deletions (random edges, edges of
  degree-1 vertices -- a move-down to unreachable on every root -- and edges
  of a root) -- followed by a comparison of all 1024 roots with the oracle's
  static recompute on the final graph (incremental = static recompute
  exactly, the reference's own property), 128 roots at a time.
* 64 R-MAT graphs of scales 10..16, K = min(|V|, 128), 512 insertions each,
  in tuned group batches of 16 per graph: every member against its own
  oracle recompute.
* Chung-Lu n = 40,000, K = 256: all 4,096 insertions in captured device
  batches of 64, against the incremental oracle every 512 insertions, then
  one call of 32 deletions (move-down) against the oracle.
* Serving: the 8 smallest of the 16 configured serving graphs (K = 512),
  Poisson arrivals: every graph's state in the mix equals its state alone,
  and both equal the oracle recompute.

dist is compared on every vertex (unreachable sets equal), sigma bit-exact
where reachable, BC within |a-b| <= 1e-9 * max(|b|, 1).
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from _util import INF32, assert_bc, assert_levels, assert_sigma, widen_dist
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

THREADS = os.cpu_count() or 1


def _check_rows_vs_static(port_lib, g2, roots, dist_rows, sigma_rows):
    """Oracle static recompute on the updated graph g2 for `roots`; the GPU's
    rows of those roots must match.  Returns the oracle's BC partial over
    these roots."""
    o = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots, nthreads=THREADS)
    o.static()
    lv = o.level()
    assert_levels(widen_dist(dist_rows), lv)
    assert_sigma(sigma_rows, o.sigma(), lv)
    bc = o.bc().copy()
    o.close()
    return bc


def test_rmat20_k1024_bench_path_vs_oracle(sbc_lib, port_lib):
    torch = pytest.importorskip("torch")
    B = 256
    train, extra = 16384, 2048
    g = G.rmat(20, 16, seed=3)
    roots = G.pick_roots(g.nv, 1024, 3)
    ins = G.rmat_insertions(g, 20, train + B + extra, seed=3)  # the benchmark's stream prefix
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    dg.reserve(ins)
    f.static_init()
    d = torch.tensor(ins, dtype=torch.int32, device="cuda")
    du, dv = d[:, 0].contiguous(), d[:, 1].contiguous()
    # cost-model training data from the first 16,384 insertions (static schedule)
    f.cost_log_start(min(train * len(roots), 1 << 26))
    for s in range(0, train, B):
        f.insert_device(B, du[s:].data_ptr(), dv[s:].data_ptr())
    f.sync()
    assert f.cost_log_stop() > 0
    f.train_cost_model(epochs=4, batch=4096, lr=2e-3, val_frac=0.1, seed=1)
    f.set_schedule(native.DeviceForest.SCHED_MODEL)
    # the tuner applies one batch after timing it under every shape
    f.autotune(ins[train:train + B], reps=1)
    for s in range(train + B, train + B + extra, B):
        f.insert_device(B, du[s:].data_ptr(), dv[s:].data_ptr())
    f.sync()
    g2 = G.insert_edges(g, ins)
    # deletions at full size, in one call
    E = G.edge_list(g2)
    rng = np.random.default_rng(29)
    deg2 = np.diff(g2.off)
    rows = f.dist(0, 8)
    row0 = rows[np.argmax((rows != INF32).sum(axis=1))]  # a root in the giant component
    leaf = E[((deg2[E[:, 0]] == 1) | (deg2[E[:, 1]] == 1)) & (row0[E[:, 0]] != INF32)]
    at_root = E[(E[:, 0] == roots[0]) | (E[:, 1] == roots[0])]
    dels = np.unique(np.concatenate([E[rng.choice(len(E), 24, replace=False)],
                                     leaf[rng.choice(len(leaf), 6, replace=False)], at_root[:2]]), axis=0)
    st = f.delete(dels)
    assert st["inserted"] == len(dels) and st["case2"] >= 1024 and st["case1"] > 0
    g2 = G.delete_edges(g2, dels)
    bc_ref = np.zeros(g.nv, dtype=np.float64)
    for r0 in range(0, len(roots), 128):
        bc_ref += _check_rows_vs_static(port_lib, g2, roots[r0:r0 + 128], f.dist(r0, 128), f.sigma(r0, 128))
    assert_bc(f.bc(), bc_ref, "rmat20 K=1024 bc vs oracle")
    f.close()
    dg.close()


def test_group64_full_size_per_graph_vs_oracle(sbc_lib, port_lib):
    B = 16
    specs = G.rmat_group(insertions=512)
    objs = []
    for g, roots, ins, _ in specs:
        dg = native.DeviceGraph(g.nv, g.off, g.adj)
        f = native.DeviceForest(dg, roots, workers=1)
        dg.reserve(ins)
        f.static_init()
        objs.append((dg, f))
    grp = native.DeviceGroup([f for _, f in objs])

    def batches(s):
        return [ins[s * B:(s + 1) * B] for _, _, ins, _ in specs]

    grp.autotune(batches(0), reps=1)
    for s in range(1, 512 // B):
        grp.insert(batches(s))
    all_bc = grp.bc()
    passed = 0
    for i, ((g, roots, ins, sc), (dg, f)) in enumerate(zip(specs, objs)):
        g2 = G.insert_edges(g, ins)
        o = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots, nthreads=THREADS)
        o.static()
        lv = o.level()
        assert_levels(f.level64(), lv)
        assert_sigma(f.sigma(), o.sigma(), lv)
        assert_bc(all_bc[i], o.bc(), f"group member {i} (scale {sc}) bc")
        o.close()
        passed += 1
    assert passed == 64
    grp.close()
    for dg, f in objs:
        f.close()
        dg.close()


def test_chunglu40k_all_insertions_captured_vs_oracle(sbc_lib, port_lib):
    torch = pytest.importorskip("torch")
    B = 64
    g, roots, ins = G.workload("chunglu40k")
    assert len(ins) == 4096
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    dg.reserve(ins)
    f.static_init()
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=THREADS)
    o.static()
    d = torch.tensor(ins, dtype=torch.int32, device="cuda")
    du, dv = d[:, 0].contiguous(), d[:, 1].contiguous()
    f.autotune(ins[:B], reps=1)  # first batch through the tuner, as the benchmark does
    for s in range(B, len(ins), B):
        f.insert_device(B, du[s:].data_ptr(), dv[s:].data_ptr())
        if (s + B) % 512 == 0:
            for u, v in ins[s + B - 512:s + B]:
                o.insert(int(u), int(v))
            lv = o.level()
            assert_levels(f.level64(), lv)
            assert_sigma(f.sigma(), o.sigma(), lv)
            assert_bc(f.bc(), o.bc(), f"chunglu40k bc after {s + B} insertions")
    g2 = G.insert_edges(g, ins)
    E = G.edge_list(g2)
    dels = E[np.random.default_rng(31).choice(len(E), 32, replace=False)]
    st = f.delete(dels)
    assert st["inserted"] == 32 and st["case2"] > 0
    for u, v in dels:
        assert o.delete(int(u), int(v))
    lv = o.level()
    assert_levels(f.level64(), lv)
    assert_sigma(f.sigma(), o.sigma(), lv)
    assert_bc(f.bc(), o.bc(), "chunglu40k bc after 32 deletions")
    o.close()
    f.close()
    dg.close()


def test_serving_eight_smallest_mix_equals_alone_and_oracle(sbc_lib, port_lib):
    graphs = G.serving_graphs(only=range(8))
    gid, pairs, t = G.poisson_trace(graphs, 4000, 50000.0, seed=11)
    srv = native.DeviceServer(budget_bytes=150 << 30, max_batch=1024)
    ids = [srv.add_graph(g, roots) for g, roots in graphs]
    srv.play(gid, pairs, t)
    srv.drain()
    mixed = [srv.read(i) for i in ids]
    st = srv.stats()
    assert st["completed"] == len(gid) and st["batches"] < len(gid)
    srv.close()
    for i, (g, roots) in enumerate(graphs):
        mine = pairs[gid == i]
        dg = native.DeviceGraph(g.nv, g.off, g.adj)
        f = native.DeviceForest(dg, roots)
        f.static_init()
        for s in range(0, len(mine), 64):
            f.insert(mine[s:s + 64])
        d, s_, b = mixed[i]
        np.testing.assert_array_equal(d, f.dist())
        np.testing.assert_array_equal(s_, f.sigma())
        assert_bc(b, f.bc(), f"serving graph {i}: mix vs alone")
        f.close()
        dg.close()
        g2 = G.insert_edges(g, mine) if len(mine) else g
        o = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots, nthreads=THREADS)
        o.static()
        lv = o.level()
        assert_levels(widen_dist(d), lv)
        assert_sigma(s_, o.sigma(), lv)
        assert_bc(b, o.bc(), f"serving graph {i}: mix vs oracle")
        o.close()
