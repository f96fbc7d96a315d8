"""CPU tests: the oracle (C restatement of the reference) is pinned against the
golden vectors produced by the unmodified reference, against networkx, and
against its own static recompute; the workload generators are checked."""
import numpy as np
import pytest

from _util import (BC_RTOL, INF64, assert_bc, assert_levels, assert_sigma, bc_err, golden_cases,
                   load_golden)
from streamingbc_gb300 import graphs as G


@pytest.mark.parametrize("case", golden_cases())
def test_port_matches_reference_golden(port_lib, case):
    z = load_golden(case)
    o = port_lib.PortOracle(int(z["nv"]), z["off"], z["adj"], z["roots"], nthreads=2)
    o.static()
    assert_levels(o.level(), z["level0"])
    assert_sigma(o.sigma(), z["sigma0"], z["level0"])
    assert_bc(o.bc(), z["bc0"], "static bc")
    for i, (u, v) in enumerate(z["ins"]):
        o.insert(int(u), int(v))
        c = o.counters()
        assert [c["vertices"], c["edges"], c["case1"], c["case2"]] == z["counters"][i].tolist(), f"counters at {i}"
        assert bc_err(o.bc(), z["bc_trace"][i]) <= BC_RTOL, f"bc after insertion {i}"
    assert_levels(o.level(), z["level1"])
    assert_sigma(o.sigma(), z["sigma1"], z["level1"])
    assert_bc(o.bc(), z["bc1"], "final bc")
    o.close()


def test_exact_bc_is_twice_networkx(port_lib):
    nx = pytest.importorskip("networkx")
    z = load_golden("karate")
    g = nx.Graph()
    g.add_nodes_from(range(int(z["nv"])))
    src = np.repeat(np.arange(int(z["nv"])), np.diff(z["off"]))
    g.add_edges_from(zip(src.tolist(), z["adj"].tolist()))
    o = port_lib.PortOracle(int(z["nv"]), z["off"], z["adj"], z["roots"], nthreads=1)
    o.static()
    ref = nx.betweenness_centrality(g, normalized=False)
    assert_bc(o.bc(), 2.0 * np.array([ref[i] for i in range(int(z["nv"]))]))
    o.close()


@pytest.mark.parametrize("seed,n,m,k,comps", [(5, 300, 900, 40, 1), (6, 400, 250, 400, 0), (7, 256, 2000, 256, 1)])
def test_incremental_equals_static_recompute(port_lib, seed, n, m, k, comps):
    g = G.er(n, m, seed)
    roots = G.pick_roots(g.nv, k, seed)
    ins = G.uniform_insertions(g, 40, seed)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=4)
    o.static()
    for u, v in ins:
        o.insert(int(u), int(v))
    g2 = G.insert_edges(g, ins)
    s = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots, nthreads=4)
    s.static()
    assert_levels(o.level(), s.level())
    assert_sigma(o.sigma(), s.sigma(), s.level())
    assert_bc(o.bc(), s.bc())
    o.close()
    s.close()


def test_port_matches_compiled_reference_random(port_lib):
    if not port_lib.ref_available():
        pytest.skip("reference harness not built here")
    g = G.rmat(10, 6, seed=9)
    roots = G.pick_roots(g.nv, 48, 9)
    ins = G.rmat_insertions(g, 10, 40, seed=9)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots, nthreads=3)
    r = port_lib.RefOracle(g.nv, g.off, g.adj, roots, nthreads=3)
    o.static()
    r.static()
    for u, v in ins:
        o.insert(int(u), int(v))
        r.insert(int(u), int(v))
        assert o.counters() == r.counters()
    lv, sg, _, bc = r.dump()
    r.close()
    assert_levels(o.level(), lv)
    assert_sigma(o.sigma(), sg, lv)
    assert_bc(o.bc(), bc)
    o.close()


def test_oracle_deletion_is_static_recompute(port_lib):
    """PortOracle.delete = a fresh static init of the graph without the edge."""
    g = G.er(80, 240, seed=4)
    roots = G.pick_roots(g.nv, g.nv, 4)
    src = np.repeat(np.arange(g.nv), np.diff(g.off))
    edges = [(int(a), int(b)) for a, b in zip(src, g.adj) if a < b]
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    gone = edges[:10]
    for u, v in gone:
        assert o.delete(u, v)
    assert not o.delete(*gone[0])  # already removed
    rest = np.asarray([e for e in edges if e not in gone])
    g2 = G.from_edges(g.nv, rest[:, 0], rest[:, 1])
    o2 = port_lib.PortOracle(g2.nv, g2.off, g2.adj, roots)
    o2.static()
    assert_levels(o.level(), o2.level())
    assert_sigma(o.sigma(), o2.sigma(), o2.level())
    assert_bc(o.bc(), o2.bc())
    o.close()
    o2.close()


def test_reference_deletion_disagrees_with_recompute(port_lib):
    """The reference's deleteEdgeStreamingBC (src/streamingbc.c:258-416, with
    moveDownTreeBrandes, src/streamingbc_internal.c:880-1401) does not end in
    the state of the modified graph: on ER 200/800, deleting (48,122) leaves
    vertex 84 of root 140 at level 4 with sigma 10, where a recomputation has
    level 3, sigma 1.  Deletions are therefore checked against the
    recomputation, not against the reference."""
    if not port_lib.ref_available():
        pytest.skip("reference harness not built here")
    g = G.er(200, 800, seed=5)
    roots = G.pick_roots(g.nv, 200, seed=3)
    r = port_lib.RefOracle(g.nv, g.off, g.adj, roots, nthreads=1)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    r.static()
    o.static()
    r.delete(48, 122)
    assert o.delete(48, 122)
    lv, sg, _, _ = r.dump()
    i = int(np.nonzero(roots == 140)[0][0])
    assert (lv[i, 84], sg[i, 84]) == (4, 10)
    assert (o.level()[i, 84], o.sigma()[i, 84]) == (3, 1)
    r.close()
    o.close()


def _check_simple(g: G.Graph):
    src = np.repeat(np.arange(g.nv), np.diff(g.off))
    assert np.all(src != g.adj), "self loop"
    key = src * g.nv + g.adj
    assert np.unique(key).size == key.size, "multi-edge"
    rev = np.sort(g.adj * g.nv + src)
    assert np.array_equal(np.sort(key), rev), "not symmetric"


def test_generators_deterministic_and_simple():
    a = G.er(500, 2000, 3)
    b = G.er(500, 2000, 3)
    assert np.array_equal(a.off, b.off) and np.array_equal(a.adj, b.adj)
    assert a.ne == 2000
    _check_simple(a)
    r = G.rmat(10, 8, 4)
    _check_simple(r)
    assert r.nv == 1024
    c = G.chung_lu(3000, 12000, 2.5, 1.0, 100.0, seed=5)
    _check_simple(c)
    import scipy.sparse as sp
    import scipy.sparse.csgraph as csg
    m = sp.csr_matrix((np.ones(c.adj.size), c.adj, c.off), shape=(c.nv, c.nv))
    assert csg.connected_components(m, directed=False)[0] == 1


def test_insertion_streams_are_new_distinct_edges():
    g = G.er(300, 1000, 8)
    r = G.rmat(9, 8, 1)
    for graph, ins in ((g, G.uniform_insertions(g, 200, 1)), (g, G.local_insertions(g, 100, 2)),
                       (r, G.rmat_insertions(r, 9, 100, 3))):
        keys = set(graph.edge_keys().tolist())
        seen = set()
        for u, v in ins.tolist():
            assert u != v
            assert u * graph.nv + v not in keys and v * graph.nv + u not in keys
            k = (min(u, v), max(u, v))
            assert k not in seen
            seen.add(k)
    loc = G.local_insertions(g, 100, 2, frac_local=1.0)
    assert len(loc) == 100


def test_pick_roots():
    assert np.array_equal(G.pick_roots(10, 10, 0), np.arange(10))
    r = G.pick_roots(1000, 100, 3)
    assert np.unique(r).size == 100 and r.min() >= 0 and r.max() < 1000
    with pytest.raises(ValueError):
        G.pick_roots(5, 6, 0)


def test_oracle_after_deletions_is_twice_networkx(port_lib):
    """Independent check of the deletion oracle: exact BC (all roots) after
    deletions that also cut vertices off equals 2 x networkx's betweenness of
    the modified graph."""
    nx = pytest.importorskip("networkx")
    g = G.er(120, 260, seed=9)
    E = G.edge_list(g)
    deg = np.diff(g.off)
    leaf = E[(deg[E[:, 0]] == 1) | (deg[E[:, 1]] == 1)][:3]
    dels = np.concatenate([E[np.random.default_rng(9).choice(len(E), 12, replace=False)], leaf])
    dels = np.unique(dels, axis=0)
    o = port_lib.PortOracle(g.nv, g.off, g.adj, np.arange(g.nv))
    o.static()
    for u, v in dels:
        assert o.delete(int(u), int(v))
    h = nx.Graph()
    h.add_nodes_from(range(g.nv))
    keep = set(map(tuple, E.tolist())) - set(map(tuple, dels.tolist()))
    h.add_edges_from(keep)
    ref = nx.betweenness_centrality(h, normalized=False)
    assert_bc(o.bc(), 2.0 * np.array([ref[i] for i in range(g.nv)]))
    o.close()
