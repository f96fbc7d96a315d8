"""Root sharding over processes (CPU, gloo): a forest split by roots across
ranks, with the graph replicated and one BC reduce, ends in the state of the
unsharded forest after insertions and deletions (levels/sigma exact, BC within
1e-9 relative)."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from _util import assert_bc, assert_levels, assert_sigma
from streamingbc_gb300.sharding import shard_roots


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shard_roots_partitions_in_order():
    roots = np.arange(10) * 3
    parts = [shard_roots(roots, r, 3) for r in range(3)]
    assert sorted(np.concatenate(parts).tolist()) == roots.tolist()
    assert parts[1].tolist() == [3, 12, 21]
    with pytest.raises(ValueError):
        shard_roots(roots, 3, 3)


@pytest.mark.parametrize("name", ["rmat", "er"])
def test_two_rank_sharded_forest_equals_unsharded(port_lib, tmp_path, name):
    import torch.multiprocessing as mp
    import _shard_worker as W
    world = 2
    mp.start_processes(W.run, args=(world, _free_port(), name, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    z = np.load(tmp_path / f"{name}_{world}.npz")
    g, roots, ins = W.case(name)
    ref = W.OracleForest(g, roots)
    ref.insert(ins)
    ref.delete(W.deletions(name))
    assert_levels(z["lv"], ref.level64())
    assert_sigma(z["sg"], ref.sigma(), ref.level64())
    assert_bc(z["bc"], ref.bc())
