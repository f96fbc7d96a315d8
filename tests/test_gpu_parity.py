"""GPU parity tests: the sm_103a kernels, called through the C-ABI, against the
golden vectors of the unmodified reference and against the oracle.

Bar: dist and sigma bit-exact (unreachable sets equal), BC within
|a-b| <= 1e-9*max(|b|,1) in FP64, traversal counters equal to the reference's.
"""
import numpy as np
import pytest

from _util import (BC_RTOL, assert_bc, assert_levels, assert_sigma, bc_err, golden_cases, load_golden,
                   widen_dist)
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu


def make(g_nv, off, adj, roots, workers=0):
    dg = native.DeviceGraph(g_nv, off, adj)
    f = native.DeviceForest(dg, roots, workers=workers)
    return dg, f


def check_state(f, lv, sg, bc, delta=None):
    assert_levels(f.level64(), lv)
    assert_sigma(f.sigma(), sg, lv)
    assert_bc(f.bc(), bc)


@pytest.mark.parametrize("case", golden_cases())
def test_static_matches_reference(sbc_lib, case):
    z = load_golden(case)
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"])
    f.static_init()
    check_state(f, z["level0"], z["sigma0"], z["bc0"])
    f.close()
    dg.close()


@pytest.mark.parametrize("case", golden_cases())
def test_each_insertion_matches_reference(sbc_lib, case):
    """One insertion per call (the plain path), BC compared after every one,
    counters compared with the reference's per-insertion counters."""
    z = load_golden(case)
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"])
    f.static_init()
    f.counters()
    for i, (u, v) in enumerate(z["ins"]):
        st = f.insert([(u, v)])
        assert st["inserted"] == 1
        got = [st["vertices"], st["edges"], st["case1"], st["case2"]]
        assert got == z["counters"][i].tolist(), f"counters after insertion {i}: {got} vs {z['counters'][i]}"
        assert bc_err(f.bc(), z["bc_trace"][i]) <= BC_RTOL, f"bc after insertion {i}"
    check_state(f, z["level1"], z["sigma1"], z["bc1"])
    f.close()
    dg.close()


@pytest.mark.parametrize("case", golden_cases())
@pytest.mark.parametrize("batch", [7, 64])
def test_batched_insertions_match_reference(sbc_lib, case, batch):
    """Insertions applied in batches (one persistent launch per batch, each root
    applies the batch in order) end in the reference's state."""
    z = load_golden(case)
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"])
    f.static_init()
    ins = z["ins"]
    for s in range(0, len(ins), batch):
        st = f.insert(ins[s:s + batch])
        assert st["inserted"] == len(ins[s:s + batch])
        last = min(s + batch, len(ins)) - 1
        assert bc_err(f.bc(), z["bc_trace"][last]) <= BC_RTOL
    check_state(f, z["level1"], z["sigma1"], z["bc1"])
    f.close()
    dg.close()


def test_every_launch_shape_same_result(sbc_lib):
    """Results do not depend on the update kernel's launch shape."""
    import ctypes
    n = ctypes.c_int()
    assert sbc_lib.sbc_update_variant_count(ctypes.byref(n)) == 0 and n.value >= 1
    z = load_golden("rmat9")
    for v in range(n.value):
        dg = native.DeviceGraph(int(z["nv"]), z["off"], z["adj"])
        f = native.DeviceForest(dg, z["roots"], variant=v)
        f.static_init()
        for s in range(0, len(z["ins"]), 16):
            f.insert(z["ins"][s:s + 16])
        check_state(f, z["level1"], z["sigma1"], z["bc1"])
        f.close()
        dg.close()


def test_deep_levels_use_exact_fallback(sbc_lib, port_lib):
    """A 600-vertex path: levels >= 254 do not fit the one-byte distance shadow
    and must be read from the int32 distances; shortcuts then move long
    stretches up by hundreds of levels."""
    n = 600
    a = np.arange(n - 1)
    g = G.from_edges(n, a, a + 1)
    roots = np.array([0, 1, 299, 599], dtype=np.int64)
    ins = np.array([(0, 400), (100, 550), (250, 260), (5, 590), (300, 310), (0, 599)], dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=2)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    check_state(f, o.level(), o.sigma(), o.bc())
    for u, v in ins:
        o.insert(int(u), int(v))
        f.insert([(u, v)])
        check_state(f, o.level(), o.sigma(), o.bc())


def test_hub_parents_direct_probe_scan_and_pull(sbc_lib, port_lib):
    """Roots of degree 1-2 above hubs: level-1 contributions go straight to the
    root, level-2 hubs find their parents by binary search in their sorted
    adjacency (and through the unsorted tail that insertions append), smaller
    level-2 vertices scan, and other roots pull.  State checked against the
    oracle after every insertion."""
    rng = np.random.default_rng(17)
    n = 3000
    us, vs = [0, 0], [1, 2]
    for h in (1, 2):                       # two hubs under root 0
        nb = rng.choice(np.arange(3, 1500), size=700, replace=False)
        us += [h] * nb.size
        vs += nb.tolist()
    nb = rng.choice(np.arange(1500, n), size=1200, replace=False)
    us += [3] * nb.size                    # a level-2 hub with a level-3 fan
    vs += nb.tolist()
    extra = rng.integers(3, n, size=(1500, 2))
    us += extra[:, 0].tolist()
    vs += extra[:, 1].tolist()
    g = G.from_edges(n, np.array(us), np.array(vs))
    roots = np.array([0, 4, 1601, 2999, 1, 3], dtype=np.int64)
    ins = [(1, 2999), (3, 1), (2, 1700), (0, 5), (1, 1800), (1, 1801), (3, 4), (2, 2500), (10, 11), (1, 1999)]
    ins = np.array([p for p in ins if p[1] not in set(g.adj[g.off[p[0]]:g.off[p[0] + 1]].tolist())], dtype=np.int64)
    ins = np.concatenate([ins, G.uniform_insertions(g, 30, seed=5)])
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=2)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    check_state(f, o.level(), o.sigma(), o.bc())
    for u, v in ins:
        o.insert(int(u), int(v))
        st = f.insert([(u, v)])
        c = o.counters()
        assert (st["vertices"], st["edges"]) == (c["vertices"], c["edges"])
        check_state(f, o.level(), o.sigma(), o.bc())


@pytest.mark.parametrize("workers", [1, 3])
def test_few_workers_same_result(sbc_lib, workers):
    z = load_golden("rmat9")
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"], workers=workers)
    f.static_init()
    f.insert(z["ins"])
    check_state(f, z["level1"], z["sigma1"], z["bc1"])


def test_er1024_exact_every_insertion_vs_oracle(sbc_lib, port_lib):
    """ER G(1024, 8192) seed 1, exact BC (K = 1024), 256 uniform insertions one
    at a time; full state compared with the oracle after every insertion."""
    g, roots, ins = G.workload("er1024")
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    check_state(f, o.level(), o.sigma(), o.bc())
    for i, (u, v) in enumerate(ins):
        o.insert(int(u), int(v))
        st = f.insert([(u, v)])
        c = o.counters()
        assert (st["vertices"], st["edges"], st["case1"], st["case2"]) == \
            (c["vertices"], c["edges"], c["case1"], c["case2"]), f"counters at {i}"
        assert_levels(f.level64(), o.level())
        assert_sigma(f.sigma(), o.sigma(), o.level())
        assert_bc(f.bc(), o.bc(), f"bc after insertion {i}")
    d_err = np.abs(f.delta() - o.delta()) / np.maximum(np.abs(o.delta()), 1.0)
    assert d_err.max() <= BC_RTOL


def test_chunglu_batches_vs_oracle(sbc_lib, port_lib):
    """Chung-Lu n=40000 (~176k edges, LCC), K = 256, 512 insertions (70% at BFS
    distance <= 3) in batches of 64, state checked after every batch."""
    g, roots, ins = G.workload("chunglu40k")
    ins = ins[:512]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    check_state(f, o.level(), o.sigma(), o.bc())
    for s in range(0, len(ins), 64):
        for u, v in ins[s:s + 64]:
            o.insert(int(u), int(v))
        f.insert(ins[s:s + 64])
        check_state(f, o.level(), o.sigma(), o.bc())


def test_rmat_incremental_equals_static_recompute(sbc_lib):
    """Size-independent property on R-MAT scale 16: the incremental state after
    1024 R-MAT-drawn insertions (batches of 64) equals a static recompute on
    the updated graph (dist/sigma bit-exact, BC within tolerance)."""
    g = G.rmat(16, 16, seed=3)
    roots = G.pick_roots(g.nv, 256, 3)
    ins = G.rmat_insertions(g, 16, 1024, seed=3)
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    for s in range(0, len(ins), 64):
        f.insert(ins[s:s + 64])
    g2 = G.insert_edges(g, ins)
    dg2, f2 = make(g2.nv, g2.off, g2.adj, roots)
    f2.static_init()
    for r0 in range(0, 256, 64):
        d1, d2 = f.dist(r0, 64), f2.dist(r0, 64)
        assert np.array_equal(d1, d2)
        reach = d2 != np.iinfo(np.int32).max
        assert np.array_equal(f.sigma(r0, 64)[reach], f2.sigma(r0, 64)[reach])
    assert_bc(f.bc(), f2.bc())


def test_rejects_duplicates_and_loops(sbc_lib):
    z = load_golden("er200")
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"])
    f.static_init()
    before = f.bc()
    u = int(z["adj"][0])
    existing = (0, u) if z["off"][1] > 0 else None
    pairs = [(5, 5), (0, 10**9)]
    if existing:
        pairs.append(existing)
    st = f.insert(pairs)
    assert st["inserted"] == 0 and st["invalid"] == 2 and st["duplicates"] == (1 if existing else 0)
    assert np.array_equal(f.bc(), before)
    # duplicate inside one batch: the second copy is rejected
    new = tuple(int(x) for x in z["ins"][0])
    st = f.insert([new, new[::-1]])
    assert st["inserted"] == 1 and st["duplicates"] == 1
    assert bc_err(f.bc(), z["bc_trace"][0]) <= BC_RTOL


def test_slack_repack_keeps_results(sbc_lib, port_lib):
    """Many insertions at one vertex overflow its slack and force a re-pack of
    the adjacency; results stay equal to the oracle."""
    g = G.er(400, 800, seed=12)
    roots = G.pick_roots(g.nv, 400, 0)
    hub = 7
    others = [v for v in range(g.nv) if v != hub and v not in set(g.adj[g.off[hub]:g.off[hub + 1]].tolist())]
    ins = np.array([(hub, v) for v in others[:60]], dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    for s in range(0, len(ins), 16):
        for u, v in ins[s:s + 16]:
            o.insert(int(u), int(v))
        f.insert(ins[s:s + 16])
    check_state(f, o.level(), o.sigma(), o.bc())
    assert dg.repacks() >= 1
    off, adj = dg.to_csr()
    assert off[hub + 1] - off[hub] == (g.off[hub + 1] - g.off[hub]) + 60


def test_edge_cases_isolated_root_and_tiny_graphs(sbc_lib, port_lib):
    # graph with an isolated root, a path, and insertions touching the root
    n = 12
    g = G.from_edges(n, np.array([1, 2, 3, 4, 6, 7]), np.array([2, 3, 4, 5, 7, 8]))
    roots = np.arange(n)
    ins = np.array([(0, 1), (5, 6), (0, 9), (9, 10), (3, 8), (1, 5)], dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=1)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    check_state(f, o.level(), o.sigma(), o.bc())
    for u, v in ins:
        o.insert(int(u), int(v))
        f.insert([(u, v)])
        check_state(f, o.level(), o.sigma(), o.bc())
    # single root, single vertex
    g1 = G.from_edges(1, np.array([], dtype=np.int64), np.array([], dtype=np.int64))
    dg1, f1 = make(1, g1.off, g1.adj, np.array([0]))
    f1.static_init()
    assert f1.dist().tolist() == [[0]] and f1.bc().tolist() == [0.0]


@pytest.mark.parametrize("capture", [True, False])
def test_device_batch_entry_point(sbc_lib, capture):
    """Device-resident batches of 8: with capture on, the first batch is
    captured as a CUDA graph and the next five replay it with re-pointed
    inputs; with capture off every batch is launched directly."""
    torch = pytest.importorskip("torch")
    z = load_golden("rmat9")
    dg, f = make(int(z["nv"]), z["off"], z["adj"], z["roots"])
    f.set_graph_capture(capture)
    f.static_init()
    dg.reserve(z["ins"])
    ins = torch.tensor(z["ins"], dtype=torch.int32, device="cuda")
    u = ins[:, 0].contiguous()
    v = ins[:, 1].contiguous()
    torch.cuda.synchronize()
    for s in range(0, u.numel(), 8):
        f.insert_device(min(8, u.numel() - s), u[s:].data_ptr(), v[s:].data_ptr())
    f.sync()
    check_state(f, z["level1"], z["sigma1"], z["bc1"])


def test_captured_batches_recaptured_after_repack(sbc_lib, port_lib):
    """A re-pack moves the adjacency; replayed graphs must be re-captured."""
    torch = pytest.importorskip("torch")
    g = G.er(400, 800, seed=12)
    roots = G.pick_roots(g.nv, 400, 0)
    hub = 7
    others = [w for w in range(g.nv) if w != hub and w not in set(g.adj[g.off[hub]:g.off[hub + 1]].tolist())]
    ins = np.array([(hub, w) for w in others[:48]], dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    d = torch.tensor(ins, dtype=torch.int32, device="cuda")
    u = d[:, 0].contiguous()
    v = d[:, 1].contiguous()
    torch.cuda.synchronize()
    for s in range(0, len(ins), 8):
        dg.reserve(ins[s:s + 8])          # slack of the hub runs out: re-packs happen between batches
        f.insert_device(8, u[s:].data_ptr(), v[s:].data_ptr())
        for a, b in ins[s:s + 8]:
            o.insert(int(a), int(b))
    f.sync()
    assert dg.repacks() >= 2
    check_state(f, o.level(), o.sigma(), o.bc())


@pytest.mark.parametrize("case", ["er1024"])
def test_autotune_keeps_results_and_picks_fastest(sbc_lib, port_lib, case):
    """The tuner's batch is applied exactly once (its timing runs work on
    copies), later batches run in the chosen shape, and the state matches the
    oracle after each batch; the chosen shape is the fastest one timed."""
    g, roots, ins = G.workload(case)
    ins = ins[:192]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    for s in range(0, len(ins), 64):
        for u, v in ins[s:s + 64]:
            o.insert(int(u), int(v))
        if s == 0:
            chosen, ms = f.autotune(ins[s:s + 64], reps=1)
            timed = ms >= 0
            assert timed.sum() >= 2 and timed[chosen]
            assert ms[chosen] == ms[timed].min()
            assert f.variant == chosen
        else:
            f.insert(ins[s:s + 64])
        check_state(f, o.level(), o.sigma(), o.bc())
    f.close()
    dg.close()


def test_switching_shapes_between_batches(sbc_lib, port_lib):
    """Re-sizing the worker scratch between batches (device batches replayed
    from captured graphs included) never changes results."""
    import ctypes
    import torch
    n = ctypes.c_int()
    sbc_lib.sbc_update_variant_count(ctypes.byref(n))
    g, roots, ins = G.workload("chunglu40k")
    ins = ins[:32 * n.value]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    dg.reserve(ins)
    f.static_init()
    d = torch.tensor(ins, dtype=torch.int32, device="cuda")
    u, v = d[:, 0].contiguous(), d[:, 1].contiguous()
    for k in range(n.value):
        f.set_variant(n.value - 1 - k)
        s = 32 * k
        for a, b in ins[s:s + 32]:
            o.insert(int(a), int(b))
        f.insert_device(32, u[s:].data_ptr(), v[s:].data_ptr())
        f.sync()
        check_state(f, o.level(), o.sigma(), o.bc())
    f.close()
    dg.close()


def test_rosters_on_deep_trees(sbc_lib, port_lib):
    """Roots of degree 1 in an R-MAT graph have deep trees whose hubs sit below
    small levels; their parents are found through the rosters of those levels.
    State equals the oracle after every batch, and every tracked roster holds
    exactly its level's members."""
    g = G.rmat(12, 8, seed=41)
    deg = np.diff(g.off)
    leaves = np.nonzero(deg == 1)[0]
    rng = np.random.default_rng(41)
    roots = np.unique(np.concatenate([rng.choice(leaves, 24, replace=False),
                                      G.pick_roots(g.nv, 8, seed=41)]))
    ins = G.rmat_insertions(g, 12, 256, seed=41)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    tracked = 0
    for s in range(0, len(ins), 32):
        for u, v in ins[s:s + 32]:
            o.insert(int(u), int(v))
        f.insert(ins[s:s + 32])
        check_state(f, o.level(), o.sigma(), o.bc())
        d = f.dist()
        for r in range(len(roots)):
            for lv in range(2, 16):
                ros = f.roster(r, lv)
                if ros is None:
                    continue
                tracked += 1
                assert sorted(ros.tolist()) == np.nonzero(d[r] == lv)[0].tolist(), (r, lv)
    assert tracked > 0
    f.close()
    dg.close()


def test_adjacency_lists_stay_sorted_across_batches(sbc_lib, port_lib):
    """The slots a batch appends are merged into each vertex's sorted list
    after the batch: lists stay sorted, so edge lookups never scan more than
    the current batch's appends.  A hub that takes more appends in one batch
    than one merge covers (2,048) is merged over the next batches.  The state
    stays the oracle's throughout."""
    g = G.rmat(12, 8, seed=61)
    roots = G.pick_roots(g.nv, 48, seed=61)
    hub = int(np.argmax(np.diff(g.off)))
    nbr = set(g.adj[g.off[hub]:g.off[hub + 1]].tolist())
    star = np.array([(hub, y) for y in range(g.nv) if y != hub and y not in nbr][:2601], dtype=np.int64)
    rest = G.rmat_insertions(g, 12, 300, seed=61)
    rest = np.array([(u, v) for u, v in rest.tolist() if hub not in (u, v)], dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()

    def sorted_lists():
        off, adj = dg.to_csr()
        return [v for v in range(g.nv) if np.any(np.diff(adj[off[v]:off[v + 1]]) <= 0)]

    batches = [rest[:100], star[:2600], np.concatenate([star[2600:], rest[100:200]]), rest[200:]]
    for k, batch in enumerate(batches):
        for u, v in batch:
            o.insert(int(u), int(v))
        f.insert(batch)
        check_state(f, o.level(), o.sigma(), o.bc())
        # 2,600 appends on the hub: 2,048 merged after their batch, the rest
        # after the next batch that appends to the hub
        assert sorted_lists() == ([hub] if k == 1 else [])


def test_level2_masks_follow_graph_changes(sbc_lib, port_lib):
    """Level-2 ascents of roots with at most 32 neighbours find parents from
    per-root masks kept up to date with the graph.  Insertions and deletions
    at the roots themselves (the mask is rebuilt) and at root neighbours (bits
    set and cleared), in batches and one at a time, interleaved: the state
    stays the oracle's."""
    g = G.rmat(9, 8, seed=71)
    deg = np.diff(g.off)
    roots = np.array([v for v in G.pick_roots(g.nv, 200, seed=71) if 0 < deg[v] <= 32][:48], dtype=np.int64)
    rng = np.random.default_rng(71)
    adj = {v: set(g.adj[g.off[v]:g.off[v + 1]].tolist()) for v in range(g.nv)}

    def new_edges(anchors, count):
        out = set()
        while len(out) < count:
            a = int(rng.choice(anchors))
            b = int(rng.integers(g.nv))
            if a != b and b not in adj[a] and (min(a, b), max(a, b)) not in out:
                out.add((min(a, b), max(a, b)))
        for a, b in out:
            adj[a].add(b)
            adj[b].add(a)
        return np.array(sorted(out), dtype=np.int64)

    def old_edges(anchors, count):
        out = []
        for a in rng.permutation(anchors):
            a = int(a)
            if adj[a] and len(out) < count:
                b = int(rng.choice(sorted(adj[a])))
                adj[a].discard(b)
                adj[b].discard(a)
                out.append((a, b))
        return np.array(out, dtype=np.int64)

    nbrs = np.array(sorted({int(y) for r in roots for y in adj[int(r)]}), dtype=np.int64)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg, f = make(g.nv, g.off, g.adj, roots)
    f.static_init()
    steps = [("ins", new_edges(roots[:6], 6)), ("ins", new_edges(nbrs, 40)), ("del", old_edges(nbrs, 5)),
             ("del", old_edges(roots[6:10], 3)), ("ins", np.concatenate([new_edges(roots[10:14], 4),
                                                                          new_edges(nbrs, 30)])),
             ("ins1", new_edges(nbrs, 5))]
    for kind, edges in steps:
        if kind == "del":
            for u, v in edges:
                assert o.delete(int(u), int(v))
            f.delete(edges)
        else:
            for u, v in edges:
                o.insert(int(u), int(v))
            if kind == "ins1":
                for e in edges:
                    f.insert([e])
            else:
                f.insert(edges)
        check_state(f, o.level(), o.sigma(), o.bc())


def test_device_batch_without_slack_appends_in_order(sbc_lib, port_lib):
    """Device batch (no host capacity planning, nothing reserved) that runs a
    vertex out of slack: the parallel append falls back to the in-order append,
    so the insertions at that vertex are taken in order until its slack ends
    and the later ones are refused (the next sync reports it); the state is
    that of the graph actually built, as a static recompute of it gives."""
    torch = pytest.importorskip("torch")
    g = G.er(300, 900, seed=8)
    roots = G.pick_roots(g.nv, 60, seed=8)
    hub = int(np.argmax(np.diff(g.off)))
    nbr = set(g.adj[g.off[hub]:g.off[hub + 1]].tolist()) | {hub}
    fresh = [x for x in range(g.nv) if x not in nbr][:40]
    ins = np.array([(hub, x) for x in fresh], dtype=np.int64)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    d = torch.tensor(ins, dtype=torch.int32, device="cuda")
    du, dv = d[:, 0].contiguous(), d[:, 1].contiguous()
    f.insert_device(len(ins), du.data_ptr(), dv.data_ptr())
    with pytest.raises(native.SbcError):
        f.sync()
    off, adj = dg.to_csr()
    got = set(adj[off[hub]:off[hub + 1]].tolist())
    taken = [x for x in fresh if x in got]
    assert 0 < len(taken) < len(fresh)
    assert taken == fresh[:len(taken)]  # in insertion order, none skipped
    g2 = G.from_edges(g.nv, np.repeat(np.arange(g.nv), np.diff(off)), adj)
    o = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots)
    o.static()
    assert_levels(f.level64(), o.level())
    assert_sigma(f.sigma(), o.sigma(), o.level())
    assert_bc(f.bc(), o.bc())
    o.close()
    f.close()
    dg.close()


def test_large_batch_in_order_append(sbc_lib, port_lib):
    """A batch larger than the parallel append takes (10,000 insertions, with
    repeats inside the batch and edges already present): appended in order by
    one warp; the result equals a static recompute of the graph with the new
    edges, and the counts split into inserted / duplicate as one-by-one
    appends would."""
    g = G.er(3000, 9000, seed=12)
    roots = G.pick_roots(g.nv, 64, seed=12)
    rng = np.random.default_rng(12)
    new = rng.integers(0, g.nv, size=(9000, 2))
    new = new[new[:, 0] != new[:, 1]]
    E = G.edge_list(g)
    ins = np.concatenate([new, new[:500, ::-1], E[:500]])[:10000]
    rng.shuffle(ins)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    st = f.insert(ins)
    g2 = G.insert_edges(g, ins)
    assert st["inserted"] == g2.ne - g.ne and st["inserted"] + st["duplicates"] == len(ins)
    o = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots)
    o.static()
    assert_levels(f.level64(), o.level())
    assert_sigma(f.sigma(), o.sigma(), o.level())
    assert_bc(f.bc(), o.bc())
    o.close()
    f.close()
    dg.close()
