"""Multi-forest batches (sbc_group): one launch sequence per batch over many
forests, each over its own graph.  Every member must end exactly where
per-forest updates (and the oracle) end: dist/sigma bit-exact, BC within
1e-9 relative."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from _util import assert_bc, assert_levels, assert_sigma
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu


def _members(count, lo, hi, k, nins, seed0=100):
    return G.rmat_group(count=count, scale_lo=lo, scale_hi=hi, edge_factor=8, seed0=seed0, k_max=k,
                        insertions=nins)


def _forests(specs):
    out = []
    for g, roots, _, _ in specs:
        dg = native.DeviceGraph(g.nv, g.off, g.adj)
        f = native.DeviceForest(dg, roots)
        f.static_init()
        out.append((dg, f))
    return out


def test_group_matches_oracle_per_member(sbc_lib, port_lib):
    """Six R-MAT graphs (scales 6..9, K <= 32) receive ragged batches (one
    member gets none in a step); after every group batch each member equals
    its own oracle."""
    specs = _members(6, 6, 9, 32, 48)
    fs = _forests(specs)
    orcs = []
    for g, roots, _, _ in specs:
        o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
        o.static()
        orcs.append(o)
    grp = native.DeviceGroup([f for _, f in fs])
    pos = [0] * len(specs)
    for step in range(4):
        batches = []
        for i, (_, _, ins, _) in enumerate(specs):
            n = 0 if (step == 1 and i == 2) else (16 - 2 * i if step < 3 else len(ins) - pos[i])
            n = max(0, min(n, len(ins) - pos[i]))
            b = ins[pos[i]:pos[i] + n]
            pos[i] += n
            batches.append(b)
            for u, v in b:
                orcs[i].insert(int(u), int(v))
        ms = grp.insert(batches)
        assert ms >= 0.0
        all_bc = grp.bc()  # every member's BC through one group read
        for i, (_, f) in enumerate(fs):
            assert_levels(f.level64(), orcs[i].level())
            assert_sigma(f.sigma(), orcs[i].sigma(), orcs[i].level())
            assert_bc(f.bc(), orcs[i].bc(), what=f"member {i} bc")
            np.testing.assert_array_equal(all_bc[i], f.bc())
    assert all(pos[i] == len(specs[i][2]) for i in range(len(specs)))
    grp.close()
    for dg, f in fs:
        f.close()
        dg.close()


def test_group_autotune_equals_solo_forests(sbc_lib):
    """A tuned group (first batch through the tuner) and solo forests given
    the same insertions end in the same state."""
    specs = _members(8, 7, 10, 64, 64, seed0=140)
    fs = _forests(specs)
    solo = _forests(specs)
    grp = native.DeviceGroup([f for _, f in fs])
    for s in range(0, 64, 32):
        batches = [ins[s:s + 32] for _, _, ins, _ in specs]
        if s == 0:
            chosen, ms = grp.autotune(batches, reps=1)
            assert ms[chosen] >= 0 and ms[chosen] == ms[ms >= 0].min()
            assert grp.info()["variant"] == chosen
        else:
            grp.insert(batches)
        for (_, f), b in zip(solo, batches):
            f.insert(b)
    for (_, a), (_, b) in zip(fs, solo):
        np.testing.assert_array_equal(a.dist(), b.dist())
        np.testing.assert_array_equal(a.sigma(), b.sigma())
        assert_bc(a.bc(), b.bc())
    c = grp.counters()
    assert c["vertices"] > 0
    grp.close()
    for dg, f in fs + solo:
        f.close()
        dg.close()


def test_group_argument_checks(sbc_lib):
    specs = _members(2, 6, 6, 16, 8, seed0=170)
    fs = _forests(specs)
    (dg0, f0), (dg1, f1) = fs
    lib = native.load()
    h = ctypes.c_void_p()
    same = (ctypes.c_void_p * 2)(f0.h, f0.h)
    assert lib.sbc_group_create(ctypes.byref(h), 2, same, -1) != 0
    f2 = native.DeviceForest(dg0, specs[0][1][:4])
    shared_graph = (ctypes.c_void_p * 2)(f0.h, f2.h)
    assert lib.sbc_group_create(ctypes.byref(h), 2, shared_graph, -1) != 0
    f2.close()
    grp = native.DeviceGroup([f0, f1])
    assert lib.sbc_forest_destroy(f0.h) != 0  # a member of a live group
    with pytest.raises(ValueError):
        grp.insert([specs[0][2][:2]])
    with pytest.raises(native.SbcError):
        grp.set_variant(99)
    grp.close()
    for dg, f in fs:
        f.close()
        dg.close()
