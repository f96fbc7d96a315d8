"""Forest checkpoints: a forest restored from a checkpoint (in host memory or
through a file) holds exactly the saved state and continues like the
original; both end at the oracle.  A truncated or foreign file is refused."""
from __future__ import annotations

import numpy as np
import pytest

from _util import assert_bc, assert_levels, assert_sigma
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu


def _case():
    g = G.rmat(12, 8, seed=61)
    deg = np.diff(g.off)
    leaves = np.nonzero(deg == 1)[0]
    rng = np.random.default_rng(61)
    roots = np.unique(np.concatenate([rng.choice(leaves, 16, replace=False), G.pick_roots(g.nv, 24, seed=61)]))
    ins = G.rmat_insertions(g, 12, 320, seed=61)
    return g, roots, ins


def _state(f):
    return f.dist(), f.sigma(), f.bc()


@pytest.mark.parametrize("through_file", [False, True])
def test_restored_forest_continues_like_the_original(sbc_lib, port_lib, tmp_path, through_file):
    g, roots, ins = _case()
    o = port_lib.PortOracle(g.nv, g.off, g.adj, roots)
    o.static()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    for s in range(0, 160, 40):
        f.insert(ins[s:s + 40])
    for u, v in ins[:160]:
        o.insert(int(u), int(v))
    ck = native.Checkpoint.take(f)
    info = ck.info()
    assert info["nv"] == g.nv and info["nk"] == len(roots) and info["ne"] == len(g.adj) + 2 * 160
    if through_file:
        path = str(tmp_path / "forest.sbc")
        ck.save(path)
        ck.close()
        ck = native.Checkpoint.load(path)
    d0, s0, b0 = _state(f)
    cd, cs, cb = ck.read()
    np.testing.assert_array_equal(cd, d0)
    np.testing.assert_array_equal(cs, s0)
    np.testing.assert_array_equal(cb, b0)
    dg2, f2 = ck.restore()
    np.testing.assert_array_equal(f2.roots, roots)
    d2, s2, b2 = _state(f2)
    np.testing.assert_array_equal(d2, d0)
    np.testing.assert_array_equal(s2, s0)
    np.testing.assert_array_equal(b2, b0)
    np.testing.assert_array_equal(f2.roster(0, 2) is None, f.roster(0, 2) is None)
    for s in range(160, len(ins), 40):
        f.insert(ins[s:s + 40])
        f2.insert(ins[s:s + 40])
    for u, v in ins[160:]:
        o.insert(int(u), int(v))
    for ff in (f, f2):
        assert_levels(ff.level64(), o.level())
        assert_sigma(ff.sigma(), o.sigma(), o.level())
        assert_bc(ff.bc(), o.bc())
    ck.close()
    f2.close()
    dg2.close()
    f.close()
    dg.close()


def test_bad_checkpoint_files_are_refused(sbc_lib, tmp_path):
    g, roots, ins = _case()
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    ck = native.Checkpoint.take(f)
    path = tmp_path / "forest.sbc"
    ck.save(str(path))
    raw = path.read_bytes()
    (tmp_path / "short.sbc").write_bytes(raw[:len(raw) // 2])
    (tmp_path / "foreign.sbc").write_bytes(b"NOTACKPT" + raw[8:])
    for name in ("short.sbc", "foreign.sbc", "missing.sbc"):
        with pytest.raises(native.SbcError):
            native.Checkpoint.load(str(tmp_path / name))
    ck.close()
    f.close()
    dg.close()
