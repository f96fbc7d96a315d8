"""Edge deletion on the GPU.  The state after a deletion is, by definition, a
static recompute of the modified graph; the oracle does exactly that (the
reference's own deletion path disagrees with it, see test_oracle.py)."""
from __future__ import annotations

import numpy as np
import pytest

from _util import assert_bc, assert_levels, assert_sigma
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu

MOVE_DOWN = native.DeviceForest.DELETE_MOVE_DOWN
RECOMPUTE = native.DeviceForest.DELETE_RECOMPUTE
both_modes = pytest.mark.parametrize("mode", [MOVE_DOWN, RECOMPUTE], ids=["move_down", "recompute"])


def _edges(g):
    src = np.repeat(np.arange(g.nv), np.diff(g.off))
    sel = src < g.adj
    return np.stack([src[sel], g.adj[sel]], axis=1)


def _check(f, o):
    assert_levels(f.level64(), o.level())
    assert_sigma(f.sigma(), o.sigma(), o.level())
    assert_bc(f.bc(), o.bc())


@both_modes
def test_deletions_one_at_a_time_exact_er(sbc_lib, port_lib, mode):
    """ER 200/800, exact BC (K = 200): 40 deletions, state after each."""
    g = G.er(200, 800, seed=5)
    roots = G.pick_roots(g.nv, g.nv, seed=5)
    rng = np.random.default_rng(5)
    dels = _edges(g)[rng.choice(g.ne, 40, replace=False)]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(mode)
    f.static_init()
    moved = adjacent = 0
    for u, v in dels:
        assert o.delete(int(u), int(v))
        st = f.delete([(u, v)])
        assert st["inserted"] == 1
        moved += st["case2"]
        adjacent += st["case1"]
        _check(f, o)
    assert moved > 0 and adjacent > 0  # both kinds of affected root met
    f.close()
    dg.close()


@both_modes
def test_rmat_deletions_between_insertion_batches(sbc_lib, port_lib, mode):
    """R-MAT scale 10 with degree-1 roots (rosters in use): insertion batches
    and deletions (of original and of newly inserted edges) interleaved."""
    g = G.rmat(10, 8, seed=9)
    deg = np.diff(g.off)
    rng = np.random.default_rng(9)
    roots = np.unique(np.concatenate([rng.choice(np.nonzero(deg == 1)[0], 16, replace=False),
                                      G.pick_roots(g.nv, 32, seed=9)]))
    ins = G.rmat_insertions(g, 10, 96, seed=9)
    orig = _edges(g)[rng.choice(g.ne, 48, replace=False)]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(mode)
    f.static_init()
    for k in range(3):
        batch = ins[32 * k:32 * (k + 1)]
        for u, v in batch:
            o.insert(int(u), int(v))
        f.insert(batch)
        _check(f, o)
        dels = np.concatenate([orig[16 * k:16 * (k + 1)], batch[:4]])
        for u, v in dels:
            o.delete(int(u), int(v))
        f.delete(dels)
        _check(f, o)
    f.close()
    dg.close()


def test_absent_and_invalid_deletions(sbc_lib, port_lib):
    g = G.er(100, 300, seed=2)
    roots = G.pick_roots(g.nv, 20, seed=2)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    before = (f.dist().copy(), f.sigma().copy(), f.bc().copy())
    present = set(map(tuple, _edges(g).tolist()))
    absent = next((u, v) for u in range(100) for v in range(u + 1, 100) if (u, v) not in present)
    st = f.delete([absent, (3, 3), (-1, 5), (7, 10 ** 6)])
    assert st["inserted"] == 0 and st["duplicates"] == 1 and st["invalid"] == 3
    np.testing.assert_array_equal(f.dist(), before[0])
    np.testing.assert_array_equal(f.sigma(), before[1])
    np.testing.assert_array_equal(f.bc(), before[2])
    f.close()
    dg.close()


def test_caller_removes_then_updates(sbc_lib, port_lib):
    """The drop-in order: the caller removes both directions
    (stinger_remove_edge x2), then asks for the update."""
    g = G.er(150, 500, seed=3)
    roots = G.pick_roots(g.nv, 40, seed=3)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(MOVE_DOWN)
    f.static_init()
    for u, v in _edges(g)[:20]:
        assert dg.remove_directed(u, v) == 1 and dg.remove_directed(v, u) == 1
        assert dg.remove_directed(u, v) == 0
        f.update_deleted(u, v)
        o.delete(int(u), int(v))
        _check(f, o)
    f.close()
    dg.close()


def test_rmat16_deletions_equal_static_recompute(sbc_lib):
    """R-MAT 16, K = 256: 96 deletions then a fresh static init of the final
    graph gives the same state (size-independent property)."""
    g = G.rmat(16, 16, seed=3)
    roots = G.pick_roots(g.nv, 256, seed=3)
    rng = np.random.default_rng(3)
    dels = _edges(g)[rng.choice(g.ne, 96, replace=False)]
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    st = f.delete(dels)
    assert st["inserted"] == 96
    keep = set(map(tuple, dels.tolist()))
    e = [(a, b) for a, b in _edges(g).tolist() if (a, b) not in keep]
    e = np.asarray(e, dtype=np.int64)
    g2 = G.from_edges(g.nv, e[:, 0], e[:, 1])
    dg2 = native.DeviceGraph(g2.nv, g2.off, g2.adj)
    f2 = native.DeviceForest(dg2, roots)
    f2.static_init()
    np.testing.assert_array_equal(f.dist(), f2.dist())
    reach = f2.dist() != np.iinfo(np.int32).max
    np.testing.assert_array_equal(f.sigma()[reach], f2.sigma()[reach])
    assert_bc(f.bc(), f2.bc())
    for x in (f, f2):
        x.close()
    dg.close()
    dg2.close()


@both_modes
def test_bridge_deletions_many_roots(sbc_lib, port_lib, mode):
    """A random tree plus a few chords: deleting a bridge leaves the deeper
    endpoint without a parent for most roots, so one deletion moves many roots'
    subtrees down at once (cutting them off the root), or recomputes them."""
    rng = np.random.default_rng(12)
    n = 300
    par = np.array([rng.integers(0, i) for i in range(1, n)])
    tree = np.stack([par, np.arange(1, n)], axis=1)
    chords = rng.integers(0, n, size=(40, 2))
    chords = chords[chords[:, 0] != chords[:, 1]]
    e = np.concatenate([tree, chords])
    g = G.from_edges(n, np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1]))
    roots = G.pick_roots(n, 120, seed=12)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(mode)
    f.static_init()
    most = 0
    for u, v in list(tree[rng.choice(len(tree), 6, replace=False)]) + list(_edges(g)[:6]):
        if not o.delete(int(u), int(v)):
            continue
        st = f.delete([(u, v)])
        most = max(most, st["case2"])
        _check(f, o)
    assert most > 16
    f.close()
    dg.close()


def test_wide_recompute_on_large_graph(sbc_lib):
    """Chung-Lu 40k: deletions of leaf edges (the leaf leaves every root's
    tree) and of random edges in one call; the result equals a static init of
    the graph without the edges."""
    g = G.chung_lu(40000, 120000, 2.5, 1.0, 200.0, seed=21)
    roots = G.pick_roots(g.nv, 48, seed=21)
    rng = np.random.default_rng(21)
    deg = np.diff(g.off)
    src = np.repeat(np.arange(g.nv), deg)
    # edges to degree-1 vertices: deleting one disconnects it for every root
    leaf_edges = np.stack([src, g.adj], axis=1)[(deg[g.adj] == 1) & (src < g.adj) | (deg[src] == 1) & (src < g.adj)]
    dels = np.concatenate([leaf_edges[rng.choice(len(leaf_edges), 4, replace=False)],
                           _edges(g)[rng.choice(g.ne, 12, replace=False)]])
    dels = np.unique(dels, axis=0)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    st = f.delete(dels)
    assert st["case2"] > 0 and st["inserted"] == len(dels)
    keep = set(map(tuple, dels.tolist()))
    e = np.asarray([(a, b) for a, b in _edges(g).tolist() if (a, b) not in keep], dtype=np.int64)
    g2 = G.from_edges(g.nv, e[:, 0], e[:, 1])
    dg2 = native.DeviceGraph(g2.nv, g2.off, g2.adj)
    f2 = native.DeviceForest(dg2, roots)
    f2.static_init()
    np.testing.assert_array_equal(f.dist(), f2.dist())
    reach = f2.dist() != np.iinfo(np.int32).max
    np.testing.assert_array_equal(f.sigma()[reach], f2.sigma()[reach])
    assert_bc(f.bc(), f2.bc())
    for x in (f, f2):
        x.close()
    dg.close()
    dg2.close()


@both_modes
def test_bridge_deletions_in_one_call(sbc_lib, port_lib, mode):
    """Deletions in one call: roots whose deeper endpoint loses its last
    parent move down, or (recompute mode) leave the call's later deletions to
    a single recompute on the final graph, while the other roots follow every
    deletion; chords first keep most roots incremental, tree edges last cut
    many roots' trees.
    The state after the call equals the oracle's, deletion by deletion."""
    rng = np.random.default_rng(13)
    n = 400
    par = np.array([rng.integers(0, i) for i in range(1, n)])
    tree = np.stack([par, np.arange(1, n)], axis=1)
    chords = rng.integers(0, n, size=(80, 2))
    chords = chords[chords[:, 0] != chords[:, 1]]
    e = np.concatenate([tree, chords])
    g = G.from_edges(n, np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1]))
    roots = G.pick_roots(n, 150, seed=13)
    edges = _edges(g)
    # chords first (most roots keep a parent), tree edges last (a bridge cuts
    # the graph, so every root recomputes from there on)
    tree_set = set(map(tuple, np.sort(tree, axis=1).tolist()))
    chord_edges = np.array([e for e in edges.tolist() if tuple(e) not in tree_set], dtype=np.int64)
    first = chord_edges[rng.choice(len(chord_edges), 20, replace=False)]
    bridges = np.sort(tree[rng.choice(len(tree), 5, replace=False)], axis=1)
    taken = set(map(tuple, first.tolist()))
    bridges = np.array([e for e in bridges.tolist() if tuple(e) not in taken], dtype=np.int64).reshape(-1, 2)
    dels = np.concatenate([first, bridges])
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    present = [bool(o.delete(int(u), int(v))) for u, v in dels]
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(mode)
    f.static_init()
    st = f.delete(dels)
    assert st["inserted"] == sum(present)
    assert st["case2"] > 0 and st["case1"] > 0
    _check(f, o)
    # and the forest goes on exactly: more deletions and insertions
    gone = set(map(tuple, dels.tolist()))
    more = np.asarray([(a, b) for a, b in edges.tolist() if (a, b) not in gone], dtype=np.int64)
    nxt = more[rng.choice(len(more), 6, replace=False)]
    for u, v in nxt:
        o.delete(int(u), int(v))
    f.delete(nxt)
    ins = G.uniform_insertions(g, 12, seed=13)
    ins = np.array([(u, v) for u, v in ins.tolist()], dtype=np.int64)
    for u, v in ins:
        o.insert(int(u), int(v))
    f.insert(ins)
    _check(f, o)
    f.close()
    dg.close()


def _two_halves(n_half, m_half, seed):
    """Two ER halves joined by one edge between their largest-degree
    vertices; returns the graph and that edge."""
    a = G.er(n_half, m_half, seed=seed)
    b = G.er(n_half, m_half, seed=seed + 1)
    ea, eb = _edges(a), _edges(b) + n_half
    bridge = (int(np.argmax(np.diff(a.off))), n_half + int(np.argmax(np.diff(b.off))))
    e = np.concatenate([ea, eb, [bridge]])
    return G.from_edges(2 * n_half, e[:, 0], e[:, 1]), bridge


def test_move_down_deep_relevels_grid_and_cycle(sbc_lib, port_lib):
    """A 24 x 24 grid (many shortest paths per vertex) joined to a cycle of
    301: deletions move whole regions down by many levels, gaining and losing
    parents on the way; every root's state after each deletion against the
    oracle."""
    w = 24
    idx = np.arange(w * w).reshape(w, w)
    grid = np.concatenate([np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1),
                           np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1)])
    c0 = w * w
    cyc = np.stack([c0 + np.arange(301), c0 + (np.arange(301) + 1) % 301], 1)
    e = np.concatenate([grid, cyc, [[idx[w // 2, w // 2], c0]]])
    n = c0 + 301
    g = G.from_edges(n, np.minimum(e[:, 0], e[:, 1]), np.maximum(e[:, 0], e[:, 1]))
    roots = np.unique(np.concatenate([G.pick_roots(n, 48, seed=31), [0, c0, c0 + 150, idx[w // 2, w // 2]]]))
    rng = np.random.default_rng(31)
    dels = np.concatenate([cyc[[0, 1, 150]], grid[rng.choice(len(grid), 30, replace=False)],
                           [[idx[w // 2, w // 2], c0]]])
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(MOVE_DOWN)
    f.static_init()
    moved = 0
    for u, v in dels:
        u, v = int(min(u, v)), int(max(u, v))
        assert o.delete(u, v)
        st = f.delete([(u, v)])
        moved += st["case2"]
        _check(f, o)
    assert moved > 0
    f.close()
    dg.close()


def test_move_down_over_cap_recomputes_small_graph(sbc_lib, port_lib):
    """Two ER halves of 1,200 vertices joined by one edge: deleting it leaves
    each root's far half (more than the move-down cap of 1,024 vertices)
    unreachable, so those roots are recomputed (a CTA per root) after the
    call; deletions before and after it in the same call are followed."""
    g, br = _two_halves(1200, 4800, seed=41)
    roots = np.unique(np.concatenate([G.pick_roots(g.nv, 40, seed=41), list(br)]))
    rng = np.random.default_rng(41)
    edges = _edges(g)
    other = edges[(edges[:, 0] != br[0]) | (edges[:, 1] != br[1])]
    pick = other[rng.choice(len(other), 8, replace=False)]
    dels = np.concatenate([pick[:4], [br], pick[4:]])
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    for u, v in dels:
        assert o.delete(int(u), int(v))
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.set_delete_mode(MOVE_DOWN)
    f.static_init()
    st = f.delete(dels)
    assert st["inserted"] == len(dels) and st["case2"] > 0
    _check(f, o)
    f.close()
    dg.close()


def test_move_down_over_cap_recomputes_large_graph(sbc_lib):
    """Two ER halves of 20,000 vertices joined by one edge (a graph of >= 32,768
    vertices): the cut roots are recomputed with the whole GPU; the result
    equals a static init of the graph without the edges."""
    g, br = _two_halves(20000, 80000, seed=43)
    roots = np.unique(np.concatenate([G.pick_roots(g.nv, 24, seed=43), list(br)]))
    rng = np.random.default_rng(43)
    edges = _edges(g)
    other = edges[(edges[:, 0] != br[0]) | (edges[:, 1] != br[1])]
    dels = np.concatenate([other[rng.choice(len(other), 6, replace=False)], [br]])
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    st = f.delete(dels)
    assert st["inserted"] == len(dels) and st["case2"] > 0
    keep = set(map(tuple, dels.tolist()))
    e = np.asarray([(a, b) for a, b in edges.tolist() if (a, b) not in keep], dtype=np.int64)
    g2 = G.from_edges(g.nv, e[:, 0], e[:, 1])
    dg2 = native.DeviceGraph(g2.nv, g2.off, g2.adj)
    f2 = native.DeviceForest(dg2, roots)
    f2.static_init()
    np.testing.assert_array_equal(f.dist(), f2.dist())
    reach = f2.dist() != np.iinfo(np.int32).max
    np.testing.assert_array_equal(f.sigma()[reach], f2.sigma()[reach])
    assert_bc(f.bc(), f2.bc())
    for x in (f, f2):
        x.close()
    dg.close()
    dg2.close()
