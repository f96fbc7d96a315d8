"""Seeded synthetic graphs, root samples and insertion streams.

These build the workloads the hot path is measured and checked on: undirected
simple graphs handed to the library as a symmetric CSR (int64 offsets and
neighbour ids, the shape of the reference's ``csrGraph``,
src/streamingbc.h:30-35), a root array (``PickRoots`` semantics: identity when
K == NV, else K distinct uniform vertices, src/sbcMain_utils.c:425-456) and a
stream of insertions of edges that are not yet in the graph (the precondition
of ``insertEdgeStreamingBC``, src/sbcMain_utils.c:458-471).

Workloads (sizes as named by the benchmark configurations):
  * ``er``        Erdos-Renyi G(n, m), no loops or multi-edges.
  * ``chung_lu``  Chung-Lu graph with power-law expected degrees, largest
                  connected component kept and relabelled 0..n'-1.
  * ``rmat``      R-MAT(scale, edge factor, a, b, c, d), symmetrised, loops and
                  duplicates dropped; isolated vertices are kept.
Everything is numpy-only and deterministic in the seed.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Graph:
    """Undirected simple graph as a symmetric CSR (both directions stored)."""

    nv: int
    off: np.ndarray  # int64 [nv+1]
    adj: np.ndarray  # int64 [off[nv]]

    @property
    def ne(self) -> int:
        """Number of undirected edges."""
        return int(self.off[-1]) // 2

    def degrees(self) -> np.ndarray:
        return np.diff(self.off)

    def edge_keys(self) -> np.ndarray:
        """Sorted int64 keys u*nv+v of every stored directed edge."""
        src = np.repeat(np.arange(self.nv, dtype=np.int64), np.diff(self.off))
        keys = src * self.nv + self.adj
        keys.sort()
        return keys


def from_edges(nv: int, u: np.ndarray, v: np.ndarray) -> Graph:
    """Symmetric CSR from an undirected edge list; drops loops and duplicates."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    keep = u != v
    u, v = u[keep], v[keep]
    lo = np.minimum(u, v)
    hi = np.maximum(u, v)
    key = _sorted_unique(lo * nv + hi)
    lo, hi = key // nv, key % nv
    both = np.concatenate([key, hi * nv + lo])  # (u,v) and (v,u) as src*nv+dst
    both.sort()
    src = both // nv
    dst = both - src * nv
    off = np.zeros(nv + 1, dtype=np.int64)
    off[1:] = np.cumsum(np.bincount(src, minlength=nv))
    return Graph(nv, off, dst.astype(np.int64))


def _sorted_unique(keys: np.ndarray) -> np.ndarray:
    """Sorted distinct values (sort + neighbour compare)."""
    k = np.sort(keys)
    if k.size == 0:
        return k
    m = np.empty(k.size, dtype=bool)
    m[0] = True
    np.not_equal(k[1:], k[:-1], out=m[1:])
    return k[m]


def _unique_in_order(keys: np.ndarray) -> np.ndarray:
    """Distinct values in order of first appearance."""
    order = np.argsort(keys, kind="stable")
    k = keys[order]
    if k.size == 0:
        return k
    m = np.empty(k.size, dtype=bool)
    m[0] = True
    np.not_equal(k[1:], k[:-1], out=m[1:])
    return keys[np.sort(order[m])]


def er(n: int, m: int, seed: int) -> Graph:
    """G(n, m): m distinct undirected non-loop edges drawn uniformly."""
    rng = np.random.default_rng(seed)
    if m > n * (n - 1) // 2:
        raise ValueError("m exceeds the number of vertex pairs")
    got = np.empty(0, dtype=np.int64)
    while got.size < m:
        need = m - got.size
        a = rng.integers(0, n, size=2 * need + 16, dtype=np.int64)
        b = rng.integers(0, n, size=2 * need + 16, dtype=np.int64)
        ok = a != b
        key = np.minimum(a, b)[ok] * n + np.maximum(a, b)[ok]
        got = _unique_in_order(np.concatenate([got, key]))
    got = got[:m]
    return from_edges(n, got // n, got % n)


def largest_component(g: Graph) -> tuple[Graph, np.ndarray]:
    """Largest connected component, relabelled densely; returns (graph, old ids)."""
    import scipy.sparse as sp
    import scipy.sparse.csgraph as csg

    a = sp.csr_matrix((np.ones(g.adj.size, dtype=np.int8), g.adj, g.off), shape=(g.nv, g.nv))
    ncomp, lab = csg.connected_components(a, directed=False)
    big = np.argmax(np.bincount(lab))
    keep = np.flatnonzero(lab == big)
    remap = -np.ones(g.nv, dtype=np.int64)
    remap[keep] = np.arange(keep.size, dtype=np.int64)
    src = np.repeat(np.arange(g.nv, dtype=np.int64), np.diff(g.off))
    sel = (remap[src] >= 0) & (remap[g.adj] >= 0)
    return from_edges(keep.size, remap[src[sel]], remap[g.adj[sel]]), keep


def chung_lu_weights(n: int, m: int, gamma: float, dmin: float, dmax: float) -> np.ndarray:
    """Expected degrees w_i = dmax * (1 + i/i0)^(-1/(gamma-1)), clipped below at
    dmin, with i0 chosen so that sum(w) = 2m: a power-law degree tail of
    exponent gamma, maximum expected degree dmax and m expected edges."""
    i = np.arange(n, dtype=np.float64)
    e = -1.0 / (gamma - 1.0)

    def total(i0):
        return np.maximum(dmin, dmax * (1.0 + i / i0) ** e).sum()

    lo, hi = 1e-6, float(n) * 1e3
    if total(hi) <= 2 * m:
        i0 = hi
    else:
        for _ in range(200):
            mid = np.sqrt(lo * hi)
            if total(mid) < 2 * m:
                lo = mid
            else:
                hi = mid
        i0 = hi
    return np.maximum(dmin, dmax * (1.0 + i / i0) ** e)


def chung_lu(n: int, m: int, gamma: float, dmin: float, dmax: float, seed: int,
             lcc: bool = True) -> Graph:
    """Chung-Lu graph with expected degrees from ``chung_lu_weights``: m
    distinct edges are drawn with both endpoints sampled proportionally to w.
    With ``lcc`` the largest connected component is kept."""
    rng = np.random.default_rng(seed)
    w = chung_lu_weights(n, m, gamma, dmin, dmax)
    p = w / w.sum()
    cdf = np.cumsum(p)
    got = np.empty(0, dtype=np.int64)
    while got.size < m:
        need = m - got.size
        a = np.searchsorted(cdf, rng.random(2 * need + 16), side="right")
        b = np.searchsorted(cdf, rng.random(2 * need + 16), side="right")
        a = np.minimum(a, n - 1).astype(np.int64)
        b = np.minimum(b, n - 1).astype(np.int64)
        ok = a != b
        key = np.minimum(a, b)[ok] * n + np.maximum(a, b)[ok]
        got = _unique_in_order(np.concatenate([got, key]))
    got = got[:m]
    g = from_edges(n, got // n, got % n)
    if lcc:
        g, _ = largest_component(g)
    return g


def _rmat_pairs(scale: int, count: int, a: float, b: float, c: float,
                rng: np.random.Generator) -> tuple[np.ndarray, np.ndarray]:
    u = np.zeros(count, dtype=np.int64)
    v = np.zeros(count, dtype=np.int64)
    ab, abc = a + b, a + b + c
    for _ in range(scale):
        r = rng.random(count)
        bu = r >= ab                      # quadrants c, d set the row bit
        bv = ((r >= a) & (r < ab)) | (r >= abc)  # quadrants b, d set the column bit
        u <<= 1
        v <<= 1
        u |= bu
        v |= bv
    return u, v


def rmat(scale: int, edge_factor: int, seed: int, a: float = 0.57, b: float = 0.19,
         c: float = 0.19) -> Graph:
    """R-MAT graph: edge_factor * 2^scale draws, symmetrised and deduplicated."""
    rng = np.random.default_rng(seed)
    n = 1 << scale
    count = edge_factor * n
    us, vs = [], []
    chunk = 1 << 22
    for s in range(0, count, chunk):
        u, v = _rmat_pairs(scale, min(chunk, count - s), a, b, c, rng)
        us.append(u)
        vs.append(v)
    return from_edges(n, np.concatenate(us), np.concatenate(vs))


def pick_roots(nv: int, k: int, seed: int) -> np.ndarray:
    """Identity when k == nv, else k distinct vertices drawn uniformly."""
    if k == nv:
        return np.arange(nv, dtype=np.int64)
    if k > nv:
        raise ValueError("more roots than vertices")
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(nv, size=k, replace=False)).astype(np.int64)


def _filter_new(g: Graph, u: np.ndarray, v: np.ndarray, taken: set[int]) -> list[tuple[int, int]]:
    keys = g.edge_keys()
    lo = np.minimum(u, v)
    hi = np.maximum(u, v)
    k = lo * g.nv + hi
    pos = np.searchsorted(keys, k)
    pos = np.minimum(pos, keys.size - 1) if keys.size else pos
    exists = (keys[pos] == k) if keys.size else np.zeros(k.size, dtype=bool)
    out = []
    for uu, vv, kk, ex in zip(u.tolist(), v.tolist(), k.tolist(), exists.tolist()):
        if uu == vv or ex or kk in taken:
            continue
        taken.add(kk)
        out.append((uu, vv))
    return out


# Candidate pairs are drawn in chunks of this fixed size, so that a stream of
# `count` insertions is a prefix of the stream for any larger count.
_CHUNK = 4096


def uniform_insertions(g: Graph, count: int, seed: int) -> np.ndarray:
    """``count`` distinct uniformly random vertex pairs that are not edges."""
    rng = np.random.default_rng(seed)
    taken: set[int] = set()
    out: list[tuple[int, int]] = []
    while len(out) < count:
        u = rng.integers(0, g.nv, size=_CHUNK, dtype=np.int64)
        v = rng.integers(0, g.nv, size=_CHUNK, dtype=np.int64)
        out += _filter_new(g, u, v, taken)
    return np.asarray(out[:count], dtype=np.int64).reshape(-1, 2)


def _ball(g: Graph, src: int, radius: int) -> np.ndarray:
    """Vertices at BFS distance 2..radius from src."""
    dist = {src: 0}
    frontier = [src]
    for d in range(1, radius + 1):
        nxt = []
        for x in frontier:
            for y in g.adj[g.off[x]:g.off[x + 1]].tolist():
                if y not in dist:
                    dist[y] = d
                    nxt.append(y)
        frontier = nxt
    return np.asarray([y for y, d in dist.items() if d >= 2], dtype=np.int64)


def local_insertions(g: Graph, count: int, seed: int, frac_local: float = 0.7,
                     radius: int = 3) -> np.ndarray:
    """Non-edge insertions, ``frac_local`` of them between vertices at BFS
    distance 2..radius of each other, the rest uniform.  Order is shuffled."""
    rng = np.random.default_rng(seed)
    n_local = int(round(frac_local * count))
    taken: set[int] = set()
    out: list[tuple[int, int]] = []
    deg = g.degrees()
    while len(out) < n_local:
        u = int(rng.integers(0, g.nv))
        if deg[u] == 0:
            continue
        ball = _ball(g, u, radius)
        if ball.size == 0:
            continue
        v = int(ball[rng.integers(0, ball.size)])
        out += _filter_new(g, np.array([u]), np.array([v]), taken)
    while len(out) < count:
        need = count - len(out)
        u = rng.integers(0, g.nv, size=2 * need + 16, dtype=np.int64)
        v = rng.integers(0, g.nv, size=2 * need + 16, dtype=np.int64)
        out += _filter_new(g, u, v, taken)[:need]
    arr = np.asarray(out[:count], dtype=np.int64).reshape(-1, 2)
    return arr[rng.permutation(arr.shape[0])]


def rmat_insertions(g: Graph, scale: int, count: int, seed: int, a: float = 0.57,
                    b: float = 0.19, c: float = 0.19) -> np.ndarray:
    """New edges drawn by the same R-MAT process, filtered to non-edges."""
    rng = np.random.default_rng(seed)
    taken: set[int] = set()
    out: list[tuple[int, int]] = []
    while len(out) < count:
        u, v = _rmat_pairs(scale, _CHUNK, a, b, c, rng)
        out += _filter_new(g, u, v, taken)
    return np.asarray(out[:count], dtype=np.int64).reshape(-1, 2)


def insert_edges(g: Graph, ins: np.ndarray) -> Graph:
    """Graph with the insertion list added (for static recompute checks)."""
    src = np.repeat(np.arange(g.nv, dtype=np.int64), np.diff(g.off))
    u = np.concatenate([src, ins[:, 0]])
    v = np.concatenate([g.adj, ins[:, 1]])
    return from_edges(g.nv, u, v)


def delete_edges(g: Graph, dels: np.ndarray) -> Graph:
    """Graph with the listed undirected edges removed (absent ones ignored)."""
    src = np.repeat(np.arange(g.nv, dtype=np.int64), np.diff(g.off))
    adj = g.adj.astype(np.int64)
    d = np.asarray(dels, dtype=np.int64).reshape(-1, 2)
    gone = np.concatenate([d[:, 0] * g.nv + d[:, 1], d[:, 1] * g.nv + d[:, 0]])
    keep = ~np.isin(src * g.nv + adj, gone)
    return from_edges(g.nv, src[keep], adj[keep])


def edge_list(g: Graph) -> np.ndarray:
    """Every undirected edge once, as (u, v) with u < v."""
    src = np.repeat(np.arange(g.nv, dtype=np.int64), np.diff(g.off))
    sel = src < g.adj
    return np.stack([src[sel], g.adj[sel].astype(np.int64)], axis=1)


# --------------------------------------------------------------------------
# Named workloads (sizes as stated for each benchmark configuration).
# --------------------------------------------------------------------------

def rmat_group(count: int = 64, scale_lo: int = 10, scale_hi: int = 16, edge_factor: int = 8, seed0: int = 100,
               k_max: int = 128, insertions: int = 512):
    """Independent R-MAT graphs for multi-forest batches: graph i has a scale
    drawn uniformly from [scale_lo, scale_hi] (one generator seeded with
    seed0), edge factor `edge_factor`, seed seed0 + i, K = min(|V|, k_max)
    uniform roots and `insertions` R-MAT-drawn new edges.
    Returns a list of (graph, roots, insertions, scale)."""
    scales = np.random.default_rng(seed0).integers(scale_lo, scale_hi + 1, size=count)
    out = []
    for i, sc in enumerate(scales):
        sc = int(sc)
        g = rmat(sc, edge_factor, seed=seed0 + i)
        roots = pick_roots(g.nv, min(g.nv, k_max), seed=seed0 + i)
        out.append((g, roots, rmat_insertions(g, sc, insertions, seed=seed0 + i), sc))
    return out


def serving_graphs(count: int = 16, n_lo: float = 1e4, n_hi: float = 1e6, gamma: float = 2.3,
                   avg_degree: float = 12.0, seed0: int = 200, k: int = 512, only=None):
    """Graphs for the serving loop: Chung-Lu graph i has n_i = n_lo *
    (n_hi/n_lo)^(i/(count-1)) vertices (log-spaced), m = avg_degree * n_i / 2
    expected edges, power-law exponent gamma, expected degrees in
    [1, sqrt(2m)] (the structural cutoff), seed seed0 + i; the largest
    connected component is kept.  K = min(|V|, k) uniform roots each.
    `only` (an iterable of indices) builds just those members of the set.
    Returns a list of (graph, roots)."""
    out = []
    for i in (range(count) if only is None else only):
        n = int(round(n_lo * (n_hi / n_lo) ** (i / max(count - 1, 1))))
        m = int(round(avg_degree * n / 2))
        g = chung_lu(n, m, gamma, 1.0, float(np.sqrt(2.0 * m)), seed=seed0 + i)
        out.append((g, pick_roots(g.nv, min(g.nv, k), seed=seed0 + i)))
    return out


def poisson_trace(graphs, count: int, rate: float, seed: int):
    """`count` insertion requests arriving as a Poisson process of `rate` per
    second; each targets graph i with probability proportional to its edge
    count and is a uniformly random non-edge of that graph (distinct within
    the graph's stream).  Returns (graph ids int32, pairs [count][2] int64,
    arrival offsets in seconds)."""
    rng = np.random.default_rng(seed)
    w = np.array([g.ne for g, _ in graphs], dtype=np.float64)
    gid = rng.choice(len(graphs), size=count, p=w / w.sum()).astype(np.int32)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    pairs = np.zeros((count, 2), dtype=np.int64)
    for i, (g, _) in enumerate(graphs):
        sel = np.nonzero(gid == i)[0]
        if sel.size:
            pairs[sel] = uniform_insertions(g, sel.size, seed=seed * 1000 + i)
    return gid, pairs, t


def workload(name: str, small: bool = False):
    """(graph, roots, insertions) for a named workload.

    er1024        ER G(1024, 8192) seed 1, K = 1024 (exact), 256 uniform insertions
    chunglu40k    Chung-Lu n=40000, ~176k edges, gamma 2.5, degrees [1,300], seed 2,
                  LCC, K = 256, 4096 insertions (70% at BFS distance <= 3)
    rmat20        R-MAT scale 20, edge factor 16, seed 3, K = 1024,
                  65536 R-MAT-drawn new edges (``small`` draws 4096)
    """
    if name == "er1024":
        g = er(1024, 8192, seed=1)
        return g, pick_roots(g.nv, g.nv, seed=1), uniform_insertions(g, 256, seed=1)
    if name == "chunglu40k":
        g = chung_lu(40000, 176000, 2.5, 1.0, 300.0, seed=2)
        return g, pick_roots(g.nv, 256, seed=2), local_insertions(g, 4096, seed=2)
    if name == "rmat20":
        g = rmat(20, 16, seed=3)
        return g, pick_roots(g.nv, 1024, seed=3), rmat_insertions(g, 20, 4096 if small else 65536, seed=3)
    raise KeyError(name)
