"""Device graph build: adjacency scattered into the slack layout and every
list sorted on the device (short lists by a warp, long ones by a block, in
shared memory or, beyond 8192 entries, in global scratch), from unsorted
input; and graphs ingested from DIMACS files give the reference's results."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from _util import assert_bc, assert_levels, assert_sigma, load_golden
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu


def test_unsorted_lists_of_every_length_are_sorted(sbc_lib):
    """Hubs of 20,000 and 3,000 neighbours, a vertex of 40, and many short
    lists, each given in shuffled order: the device adjacency holds every list
    sorted and equal (as a multiset) to the input."""
    rng = np.random.default_rng(11)
    n = 30000
    us, vs = [], []
    for hub, d in ((0, 20000), (1, 3000), (2, 40)):
        nb = rng.choice(np.arange(3, n), size=d, replace=False)
        us += [hub] * d
        vs += nb.tolist()
    e = rng.integers(3, n, size=(40000, 2))
    e = e[e[:, 0] != e[:, 1]]
    us += e[:, 0].tolist()
    vs += e[:, 1].tolist()
    g = G.from_edges(n, np.array(us), np.array(vs))
    # shuffle every vertex's list
    adj = g.adj.copy()
    for v in range(n):
        seg = adj[g.off[v]:g.off[v + 1]]
        rng.shuffle(seg)
    assert not np.array_equal(adj, g.adj)
    dg = native.DeviceGraph(n, g.off, adj)
    off2, adj2 = dg.to_csr()
    np.testing.assert_array_equal(off2, g.off)
    np.testing.assert_array_equal(adj2, g.adj)  # from_edges lists are sorted
    dg.close()


def test_dimacs_graph_matches_reference_golden(sbc_lib, tmp_path):
    """karate written as DIMACS, ingested through sbc_graph_create_dimacs:
    static init with the golden roots (shifted past vertex 0) gives the
    reference's golden levels, sigma and BC."""
    from test_ingest import to_dimacs
    z = load_golden("karate")
    n0 = int(z["nv"])
    path = tmp_path / "karate.graph"
    path.write_text(to_dimacs(n0, z["off"], z["adj"]))
    dg = native.DeviceGraph.from_dimacs(str(path))
    assert dg.nv == n0 + 1
    f = native.DeviceForest(dg, z["roots"] + 1)
    f.static_init()
    assert_levels(f.level64()[:, 1:], z["level0"])
    assert_sigma(f.sigma()[:, 1:], z["sigma0"], z["level0"])
    assert_bc(f.bc()[1:], z["bc0"])
    assert f.bc()[0] == 0.0
    f.close()
    dg.close()


def test_parse_dimacs_graph_drop_in(sbc_lib, tmp_path):
    """ParseDimacsGraph: NV counts vertex 0, NE is the header's doubled, and
    the STINGER shim's graph has the file's degrees."""
    from test_ingest import to_dimacs
    z = load_golden("dolphins")
    n0 = int(z["nv"])
    path = tmp_path / "dolphins.graph"
    path.write_text(to_dimacs(n0, z["off"], z["adj"], ne_header=159))
    lib = sbc_lib
    lib.ParseDimacsGraph.argtypes = [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.ParseDimacsGraph.restype = None
    lib.stinger_outdegree.argtypes = [C.c_void_p, C.c_int64]
    lib.stinger_outdegree.restype = C.c_int64
    lib.stinger_free.argtypes = [C.c_void_p]
    lib.stinger_free.restype = C.c_void_p
    st, nv, ne = C.c_void_p(), C.c_int64(0), C.c_int64(0)
    lib.ParseDimacsGraph(str(path).encode(), C.byref(st), C.byref(nv), C.byref(ne))
    assert st.value
    assert nv.value == n0 + 1 and ne.value == 2 * 159
    deg = np.diff(z["off"])
    assert lib.stinger_outdegree(st, 0) == 0
    for u in range(n0):
        assert lib.stinger_outdegree(st, u + 1) == deg[u]
    lib.stinger_free(st)
    bad = tmp_path / "bad.graph"
    bad.write_text("2 1\n5\n")
    st2 = C.c_void_p(1)
    lib.ParseDimacsGraph(str(bad).encode(), C.byref(st2), C.byref(nv), C.byref(ne))
    assert not st2.value
