"""Serving loop: requests for several resident graphs arrive as a Poisson
process and are batched per graph.  Each graph must end exactly where its own
insertion stream applied alone ends (dist/sigma bit-exact, BC within 1e-9
relative), whatever the batching and the mix; admission keeps the admitted
footprint within the HBM budget."""
from __future__ import annotations

import numpy as np
import pytest

from _util import assert_bc
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix():
    graphs = G.serving_graphs(count=4, n_lo=1500, n_hi=6000, k=48, seed0=300)
    gid, pairs, t = G.poisson_trace(graphs, 800, 20000.0, seed=5)
    refs = []
    for i, (g, roots) in enumerate(graphs):
        dg = native.DeviceGraph(g.nv, g.off, g.adj)
        f = native.DeviceForest(dg, roots)
        f.static_init()
        mine = pairs[gid == i]
        for s in range(0, len(mine), 64):
            f.insert(mine[s:s + 64])
        refs.append((f.dist(), f.sigma(), f.bc()))
        f.close()
        dg.close()
    return graphs, gid, pairs, t, refs


def _check(state, ref):
    d, s, b = state
    rd, rs, rb = ref
    np.testing.assert_array_equal(d, rd)
    np.testing.assert_array_equal(s, rs)
    assert_bc(b, rb)


def test_alone_unbatched_equals_reference(sbc_lib, mix):
    """Graph 0 served alone one request per batch (the plain path)."""
    graphs, gid, pairs, t, refs = mix
    srv = native.DeviceServer(budget_bytes=8 << 30, max_batch=1)
    g, roots = graphs[0]
    k = srv.add_graph(g, roots)
    sel = gid == 0
    srv.play(np.zeros(int(sel.sum()), dtype=np.int32) + k, pairs[sel], t[sel] - t[sel][0])
    srv.drain()
    _check(srv.read(k), refs[0])
    st = srv.stats()
    assert st["completed"] == sel.sum() and st["batches"] == sel.sum()
    srv.close()


def test_tuned_and_model_scheduled_serving_equals_alone(sbc_lib, mix):
    """Every graph's first batch through the launch-shape tuner and its
    batches after the first 100 insertions ordered by its own trained cost
    model: each graph still ends where its stream alone ends."""
    graphs, gid, pairs, t, refs = mix
    srv = native.DeviceServer(budget_bytes=8 << 30, max_batch=64, autotune=True, train_insertions=100)
    ids = [srv.add_graph(g, roots) for g, roots in graphs]
    srv.play(gid, pairs, t)
    srv.drain()
    for i in ids:
        _check(srv.read(i), refs[i])
    assert srv.stats()["completed"] == len(gid)
    srv.close()


@pytest.mark.parametrize("max_batch,max_inflight", [(64, 0), (1, 1)])
def test_mix_equals_alone(sbc_lib, mix, max_batch, max_inflight):
    """All graphs served together, with continuous batching or one insertion
    at a time over all graphs: every graph ends where its own stream alone
    ends."""
    graphs, gid, pairs, t, refs = mix
    srv = native.DeviceServer(budget_bytes=8 << 30, max_batch=max_batch, max_inflight=max_inflight)
    ids = [srv.add_graph(g, roots) for g, roots in graphs]
    assert ids == list(range(len(graphs)))
    srv.play(gid, pairs, t)
    srv.drain()
    for i in ids:
        _check(srv.read(i), refs[i])
    st = srv.stats()
    assert st["completed"] == len(gid)
    if max_batch > 1:
        assert st["batches"] < len(gid)  # requests arriving during a batch joined the next one
    else:
        assert st["batches"] == len(gid)
    assert 0 < st["p50_us"] <= st["p99_us"] <= st["max_us"]
    assert st["throughput"] > 0
    srv.close()


def test_admission_by_hbm_budget(sbc_lib, mix):
    """Graphs are admitted in registration order while their footprints fit
    the budget; the rest wait with their requests queued and are admitted as
    earlier graphs are released.  Every graph ends at its reference."""
    graphs, gid, pairs, t, refs = mix
    probe = native.DeviceServer(budget_bytes=1 << 40, max_batch=64)
    fps = [probe.graph_info(probe.add_graph(g, roots))["footprint"] for g, roots in graphs]
    probe.close()
    budget = max(fps) + fps[0] // 2
    assert fps[0] + fps[1] + fps[2] > budget  # at most two fit at once
    srv = native.DeviceServer(budget_bytes=budget, max_batch=64)
    ids = [srv.add_graph(g, roots) for g, roots in graphs]
    srv.play(gid, pairs, t)
    waiting = list(ids)
    rounds = 0
    while waiting:
        srv.drain()
        # expected: the longest prefix of the waiting list that fits (FIFO)
        used, expect = 0, []
        for i in waiting:
            if used + fps[i] > budget:
                break
            used += fps[i]
            expect.append(i)
        states = {i: srv.graph_info(i)["state"] for i in waiting}
        assert [i for i in waiting if states[i] == "admitted"] == expect, (rounds, states)
        assert srv.stats()["bytes_admitted"] <= budget
        for i in expect:
            assert srv.graph_info(i)["completed"] == int((gid == i).sum())
            _check(srv.read(i), refs[i])
            srv.release(i)
        waiting = [i for i in waiting if i not in expect]
        rounds += 1
    assert rounds >= 2
    assert all(srv.graph_info(i)["state"] == "released" for i in ids)
    srv.close()


@pytest.mark.timeout(300)
def test_drain_waits_for_static_init_without_requests(sbc_lib, mix):
    """drain() right after registering graphs (no requests yet) returns once
    their static init is done; their state is then readable."""
    graphs, _, _, _, _ = mix
    srv = native.DeviceServer(budget_bytes=8 << 30, max_batch=64)
    ids = [srv.add_graph(g, roots) for g, roots in graphs[:2]]
    srv.drain()
    for i in ids:
        assert srv.graph_info(i)["state"] == "admitted"
        d, s, b = srv.read(i)
        assert (d[np.arange(len(graphs[i][1])), graphs[i][1]] == 0).all()  # each root at level 0
    srv.close()


@pytest.mark.timeout(300)
def test_eviction_and_restore(sbc_lib, mix):
    """A budget that holds one graph at a time: graph 0 serves the first half
    of its stream and is evicted (checkpointed into host memory), so graph 1
    is admitted; graph 0 reads back from its checkpoint, queues the second
    half meanwhile, and once graph 1 is released is restored (no static init)
    and runs what queued.  Both graphs end at their references."""
    graphs, gid, pairs, t, refs = mix
    probe = native.DeviceServer(budget_bytes=1 << 40, max_batch=64)
    fps = [probe.graph_info(probe.add_graph(g, roots))["footprint"] for g, roots in graphs[:2]]
    probe.close()
    budget = max(fps) * 3 // 2
    assert fps[0] + fps[1] > budget
    srv = native.DeviceServer(budget_bytes=budget, max_batch=64)
    a = srv.add_graph(*graphs[0])
    b = srv.add_graph(*graphs[1])
    mine_a, mine_b = pairs[gid == 0], pairs[gid == 1]
    half = len(mine_a) // 2
    for u, v in mine_a[:half]:
        srv.submit(a, int(u), int(v))
    for u, v in mine_b:
        srv.submit(b, int(u), int(v))
    srv.drain()
    assert srv.graph_info(a)["state"] == "admitted" and srv.graph_info(b)["state"] == "waiting"
    partial = srv.read(a)
    srv.evict(a)
    srv.drain()
    assert srv.graph_info(a)["state"] == "evicted"
    assert srv.graph_info(b)["state"] == "admitted"
    for x, y in zip(srv.read(a), partial):  # from the checkpoint: the state at eviction
        np.testing.assert_array_equal(x, y)
    for u, v in mine_a[half:]:
        srv.submit(a, int(u), int(v))
    srv.drain()
    assert srv.graph_info(a)["state"] == "evicted"  # does not fit beside graph 1
    _check(srv.read(b), refs[1])
    srv.release(b)
    srv.drain()
    assert srv.graph_info(a)["state"] == "admitted"
    assert srv.graph_info(a)["completed"] == len(mine_a)
    _check(srv.read(a), refs[0])
    assert srv.stats()["bytes_admitted"] <= budget
    srv.close()
