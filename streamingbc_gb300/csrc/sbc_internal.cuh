// Internal device-side definitions of the GB300 StreamingBC hot path.
//
// HBM layout (one graph, one forest):
//   adjacency  slack CSR: row[v] (int64 slot start), deg[v] live degree, cap[v],
//              deg0[v] degree when the current batch began, col[slot] int32
//              neighbour id, seq[slot] int32 global insertion sequence number of
//              slots appended by insertions (read only for slots >= deg0[v]).
//   forest     structure-of-arrays, root-major: dist[K][V] int32
//              (SBC_INF = unreachable), sigma[K][V] int64 (0 when unreachable),
//              delta[K][V] fp64, bc[V] fp64.
//   workers    per persistent-CTA scratch, V entries each: st int32 (state bits),
//              dp int64 (diffPath), acc fp64 (dependency accumulator), and three
//              int32 vertex queues (descent, ascent-up, ascent-same) plus level
//              offsets.  Scratch is reset in O(touched) after every job.
#pragma once
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#define SBC_INF 0x7fffffff

// One-byte shadow of dist, gathered by the frontier walkers (dist8[K][V]):
// 0..253 exact level, 254 = level >= 254 (read the int32 dist), 255 = unreachable.
// A root's gathered row shrinks from 4 B to 1 B per vertex, so a hub's sorted
// neighbour list touches fewer DRAM sectors and more of the row stays in L2.
#define SBC_D8_DEEP 254
#define SBC_D8_INF 255

// Two-bit shadow of dist (dist2[K][d2_words(V)] 32-bit words, 16 vertices per
// word, vertex k in bits 2*(k%16)..): dist mod 3 for a reachable vertex, 3
// when unreachable.  Every neighbour of a reachable vertex at level L sits at
// level L-1, L or L+1 (neighbours in a BFS tree differ by at most one level,
// and share the vertex's component), so the code alone tells which.  The
// walkers of the insertion update gather from it wherever the walked
// vertices of a level all sit at one known level of a consistent labelling:
// a root's gathered row is V/4 bytes (256 KB at 2^20 vertices, against 1 MB
// for the one-byte shadow), so the rows of the roots in flight on every SM
// stay in L2 and a hub's neighbour gathers stop missing to HBM.

// Worker state bits (st[]).  Low bits: descent step + 1 (0 = not a descent
// vertex).  MOVED: the vertex moved up a level.  ASC: touched by the ascent only.
#define SBC_STEP_MASK 0x03ffffff
#define SBC_MOVED 0x08000000
#define SBC_ASC 0x10000000

namespace sbc {

struct DevGraph {
    int64_t nv;
    const int64_t* row;
    const int32_t* deg;
    const int32_t* deg0;
    const int32_t* nsort;  // the first nsort[v] slots of v are sorted by neighbour id
    const int32_t* col;
    const int32_t* seq;
};

// Whether slot p is still an edge for the job with sequence g.  TOMB: a batch
// of deletions is under way, whose removed slots stay in place until it ends
// with seq = -1 - i (i = the deletion that removed them), so the job of
// deletion g skips those removed at deletions <= g.  Every other walker is
// compiled without the test.
template <bool TOMB>
__device__ __forceinline__ bool slot_live(const DevGraph& G, int64_t p, int g)
{
    if (!TOMB) return true;
    const int q = G.seq[p];
    return q >= 0 || -1 - q > g;
}

// One forest as an update launch sees it: its graph, its root-major state and
// the insertion batch staged for it (endpoints and append codes).
struct ForestSlot {
    DevGraph G;
    const int64_t* roots;
    int32_t* dist;
    uint8_t* dist8;
    uint32_t* dist2;    // [nk][d2_words(nv)] two-bit shadow
    int64_t* sigma;
    double* delta;
    double* bc;
    const int32_t* ins_u;
    const int32_t* ins_v;
    const int32_t* ins_ok;
    int nins;
    int nk;
    int32_t* lvlhist;   // [nk][kHistLevels] vertices per level (last bucket: that level and deeper), or null
    int32_t* cost_log;  // [nk][nins] touched vertices of each job (cost-model training data), or null
    int32_t* roster;    // [nk][kRosterLevels][kRosterCap] members of small levels, or null
    int32_t* roster_n;  // [nk][kRosterLevels] entries (> kRosterCap: level not tracked)
    int32_t* roster_dirty;  // [nk][kRosterLevels] 1 once an entry went stale
    const uint32_t* l2mask; // [nk][nv] level-2 parent masks (see kL1Max), or null
    const int32_t* l1cand;  // [nk][kL1Max] the root's neighbours, bit i of a mask = l1cand[i]
    const int32_t* l1n;     // [nk] their count, -1 where the root has no masks
};

// Level-2 parent masks.  The parents of a vertex x at level 2 of root r's
// tree are its neighbours at level 1, i.e. N(x) ∩ N(r) -- a relation of the
// graph alone, whatever the BFS state.  For a root with at most kL1Max
// neighbours l1cand[r][0..n), mask[r][x] holds bit i set iff l1cand[r][i] is
// adjacent to x through an edge that existed when the current batch began
// (built after static init, extended by every batch's insertions and cleared
// by deletions; rebuilt when an edge of the root itself changes).  A level-2
// ascent step then finds each vertex's parents with one load instead of
// scanning adjacency lists.
constexpr int kL1Max = 32;

// Levels tracked by the per-root level histograms (deeper levels share the last bucket).
constexpr int kHistLevels = 64;
// Rosters: per root, the members of every level 2..kRosterLevels-1 that has at
// most kRosterCap vertices.  A roster is a superset of its level (entries of
// vertices that moved to a shallower level stay until compaction; readers
// check the distance), so a vertex deep in the tree can find its parents
// among the few members of the level above by binary search in its own
// sorted adjacency instead of scanning that adjacency.
constexpr int kRosterLevels = 16;
constexpr int kRosterCap = 256;

struct Scratch {
    int32_t* st;
    int64_t* dp;
    double* acc;
    int32_t* qd;
    int32_t* qa;
    int32_t* qs;
    int32_t* lvl;
    uint32_t* bits;  // one bit per vertex: member of the level being pulled from
};

// Words of the per-worker vertex bitmap.
__host__ __device__ __forceinline__ size_t bitmap_words(int64_t nv) { return (size_t)(nv + 31) / 32 + 1; }

// Slots of one worker w inside the worker-major scratch arrays.
struct ScratchBase {
    int32_t* st;
    int64_t* dp;
    double* acc;
    int32_t* qd;
    int32_t* qa;
    int32_t* qs;
    int32_t* lvl;    // (nv + 2) per worker
    uint32_t* bits;  // bitmap_words(nv) per worker
    __device__ __forceinline__ Scratch of(int w, int64_t nv) const
    {
        Scratch s;
        size_t o = (size_t)w * (size_t)nv;
        s.st = st + o;
        s.dp = dp + o;
        s.acc = acc + o;
        s.qd = qd + o;
        s.qa = qa + o;
        s.qs = qs + o;
        s.lvl = lvl + (size_t)w * (size_t)(nv + 2);
        s.bits = bits + (size_t)w * bitmap_words(nv);
        return s;
    }
};

// Number of neighbour slots of x visible to the insertion with sequence g:
// every slot below deg0[x], then the appended slots whose seq <= g.  Slots are
// appended in sequence order, so those are a prefix of [deg0, deg): found by
// binary search (a hub can take dozens of a batch's insertions; one dependent
// load per appended slot was a long serial chain on every visit).
__device__ __forceinline__ int vis_deg(const DevGraph& G, int x, int64_t rs, int g)
{
    const int d0 = G.deg0[x];
    const int d = G.deg[x];
    if (d0 == d || g == INT_MAX) return d;
    int lo = d0, hi = d;  // first slot in [d0, d) with seq > g
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (G.seq[rs + mid] <= g) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Is y among the first vx (visible) neighbours of x, whose slots start at rx?
// Binary search of the sorted leading slots, then a scan of the appended tail.
// Adds the number of slots examined to *cost.
template <bool TOMB = false>
__device__ __forceinline__ bool has_edge(const DevGraph& G, int x, int64_t rx, int vx, int y, int g, unsigned& cost)
{
    const int ns = min(G.nsort[x], vx);
    int lo = 0, hi = ns;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int c = G.col[rx + mid];
        ++cost;
        if (c < y) lo = mid + 1;
        else if (c > y) hi = mid;
        else return slot_live<TOMB>(G, rx + mid, g);
    }
    for (int s = ns; s < vx; ++s) {
        ++cost;
        if (G.col[rx + s] == y) return slot_live<TOMB>(G, rx + s, g);
    }
    return false;
}

__device__ __forceinline__ uint8_t enc_d8(int d)
{
    return d == SBC_INF ? (uint8_t)SBC_D8_INF : (d >= SBC_D8_DEEP ? (uint8_t)SBC_D8_DEEP : (uint8_t)d);
}

// 32-bit words of one root's two-bit row.
__host__ __device__ __forceinline__ int64_t d2_words(int64_t nv) { return (nv + 15) / 16; }

__device__ __forceinline__ unsigned enc_d2(int d) { return d == SBC_INF ? 3u : (unsigned)(d % 3); }

// Level of a neighbour whose two-bit code is c, of a vertex at level Lw >= 0.
__device__ __forceinline__ int dec_d2(unsigned c, int Lw)
{
    if (c == 3u) return SBC_INF;
    const unsigned m = (unsigned)(Lw + 2) % 3u;  // code of level Lw - 1
    return Lw - 1 + (int)((c + 3u - m) % 3u);
}

// Sets vertex k's code in a two-bit row to that of level d.  Only the thread
// that owns k's new level writes k, and XOR touches k's two bits alone, so
// concurrent updates of other vertices in the same word need no lock.
__device__ __forceinline__ void set_d2(uint32_t* R, int k, int d)
{
    const int sh = (k & 15) * 2;
    const unsigned old = (R[k >> 4] >> sh) & 3u;
    const unsigned nw = enc_d2(d);
    if (old != nw) atomicXor(&R[k >> 4], (old ^ nw) << sh);
}

// Where a walker reads its neighbours' distances: the two-bit row D2 when the
// walked vertices all sit at level Lw of a consistent labelling, else the
// one-byte row D8 (falling back to the int32 row D for levels >= 254).
struct DistRow {
    const int32_t* D;
    const uint8_t* D8;
    const uint32_t* D2;  // null: gather from D8
    int Lw;
};

__device__ __forceinline__ void atomic_add_i64(int64_t* p, int64_t v)
{
    atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v));
}

// warp_reserve: the slot index in a queue whose length is the shared counter
// *cnt for each calling lane whose `take` is set (-1 for the others);
// warp_append: appends x there.  One shared atomic per warp instead
// of one per appended vertex: the lanes converged here vote with a ballot,
// the lowest taker reserves the warp's slots, and every taker writes at its
// rank among them (frontier compaction by ballot and population count).
__device__ __forceinline__ int warp_reserve(int* cnt, bool take)
{
    const unsigned act = __activemask();
    const unsigned vote = __ballot_sync(act, take);
    if (!take) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(vote) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(cnt, __popc(vote));
    base = __shfl_sync(vote, base, leader);
    return base + __popc(vote & ((1u << lane) - 1u));
}

__device__ __forceinline__ void warp_append(int* cnt, int32_t* q, int x, bool take)
{
    const int p = warp_reserve(cnt, take);
    if (p >= 0) q[p] = x;
}

// Block-wide exclusive scan of one int per thread; returns the thread's prefix
// and writes the block total to *total (all threads).
template <int NT>
__device__ __forceinline__ int block_exclusive_scan(int v, int* s_warp, int* total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < NT / 32) ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < NT / 32) s_warp[lane] = w;
    }
    __syncthreads();
    int prefix = (wid ? s_warp[wid - 1] : 0) + x - v;
    *total = s_warp[NT / 32 - 1];
    __syncthreads();
    return prefix;
}

// Shared memory used by the load-balanced frontier walker.
template <int NT>
struct LbSmem {
    int x[NT];
    int off[NT + 1];
    int64_t row[NT];
    int warp[NT / 32];
    // traversal counters of the block: vertices walked and their visible
    // degrees as the reference counts them, and adjacency slots actually scanned
    unsigned long long walked_v, walked_e, scanned_e;
};

// Edges each thread has in flight per round of the walker: the adjacency
// slots of all of them are loaded first, then all neighbour-distance gathers,
// and only then are they processed, so a thread keeps ILP (default kEdgeIlp) independent
// HBM reads outstanding instead of one.
constexpr int kEdgeIlp = 4;

// Adjacency slots of one round of a walker chunk.  A chunk's `total` edges are
// dealt out in rounds of NT * per, per = ceil(total / NT) capped at ILP: in
// each round thread t takes the `per` consecutive edges from e0 = round start +
// t * per.  Consecutive edges mostly share a source vertex, so a thread finds
// its vertex with one binary search over the chunk's offsets per round and
// then steps (a hub's adjacency costs no search per edge), while a chunk of at
// most NT edges still gives every thread one edge and no thread a serial chain
// of several.  Sets kk[u] (neighbour, -1 past the end) and jj[u] (chunk vertex)
// for u < per; j is the thread's current chunk vertex, which only moves forward.
template <int NT, int ILP, bool TOMB>
__device__ __forceinline__ void walk_fetch(const DevGraph& G, const LbSmem<NT>& sm, int cnt, int total, int e0,
                                           int per, int g, int& j, int (&kk)[ILP], int (&jj)[ILP])
{
#pragma unroll
    for (int u = 0; u < ILP; ++u) {
        const int e = e0 + u;
        kk[u] = -1;
        jj[u] = j;
        if (u < per && e < total) {
            if (sm.off[j + 1] <= e) {
                int lo = j + 1, hi = cnt - 1;
                // within a round the next edge is usually on the next vertex
                // (off[j+1] <= e < total = off[cnt] keeps j + 2 <= cnt)
                if (u > 0 && sm.off[j + 2] > e) hi = lo;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (sm.off[mid] <= e) lo = mid;
                    else hi = mid - 1;
                }
                j = lo;
            }
            jj[u] = j;
            const int64_t p = sm.row[j] + (e - sm.off[j]);
            kk[u] = G.col[p];
            if (!slot_live<TOMB>(G, p, g)) kk[u] = -1;
        }
    }
}

// Distances of the walker's neighbours kk[u] (those >= 0) into dk[u]: every
// gather of a round is issued before any is decoded.
template <int ILP>
__device__ __forceinline__ void gather_dist(const DistRow& dr, const int (&kk)[ILP], int (&dk)[ILP])
{
    if (dr.D2) {
        unsigned w[ILP];
#pragma unroll
        for (int u = 0; u < ILP; ++u) w[u] = kk[u] >= 0 ? dr.D2[kk[u] >> 4] : 0u;
#pragma unroll
        for (int u = 0; u < ILP; ++u) dk[u] = dec_d2((w[u] >> ((kk[u] & 15) * 2)) & 3u, dr.Lw);
    } else {
#pragma unroll
        for (int u = 0; u < ILP; ++u) dk[u] = kk[u] >= 0 ? (int)dr.D8[kk[u]] : 0;
#pragma unroll
        for (int u = 0; u < ILP; ++u) {
            if (dk[u] == SBC_D8_INF) dk[u] = SBC_INF;
            else if (dk[u] == SBC_D8_DEEP) dk[u] = dr.D[kk[u]];
        }
    }
}

// Edge-balanced walk over the neighbours of a vertex list given as up to two
// ranges (l1[0..n1) then l2[0..n2)).  Vertices are taken NT at a time; each
// thread runs prep(j, x, visible_degree) for its vertex, an exclusive scan of
// the visible degrees spreads the chunk's edges evenly over the block, and
// edge(j, x, k, dist[k]) runs once per visible neighbour k (slots dealt out by
// walk_fetch, a warp reading one contiguous run; the distance is gathered from
// the root's one-byte row D8, falling back to the int32 row D only for levels
// >= 254).  post(j, x) runs after the chunk's edges.  Ends with a barrier.
// REF: the walked vertices and their degrees count as traversed in the
// reference's sense (COUNT_TRAVERSALS); every walk counts its scanned slots.
template <int NT, bool REF = true, int ILP = kEdgeIlp, bool TOMB = false, class Prep, class Edge, class Post>
__device__ __forceinline__ void lb_walk(const DevGraph& G, int g, const DistRow dr,
                                        const int32_t* l1, int n1, const int32_t* l2, int n2, LbSmem<NT>& sm,
                                        Prep prep, Edge edge, Post post)
{
    const int n = n1 + n2;
    for (int base = 0; base < n; base += NT) {
        const int t = threadIdx.x;
        const int cnt = min(NT, n - base);
        int d = 0;
        if (t < cnt) {
            int idx = base + t;
            int x = idx < n1 ? l1[idx] : l2[idx - n1];
            int64_t rs = G.row[x];
            d = vis_deg(G, x, rs, g);
            sm.x[t] = x;
            sm.row[t] = rs;
            prep(t, x, d);
        }
        int total;
        int off = block_exclusive_scan<NT>(d, sm.warp, &total);
        if (t < cnt) sm.off[t] = off;
        if (t == 0) {
            sm.off[cnt] = total;
            if (REF) {
                sm.walked_v += (unsigned)cnt;
                sm.walked_e += (unsigned)total;
            }
            sm.scanned_e += (unsigned)total;
        }
        __syncthreads();
        int j = 0;  // chunk vertex of this thread's current edge; edges only move forward
        const int per = min(ILP, (total + NT - 1) / NT);
        for (int e0 = t * per; e0 < total; e0 += NT * per) {
            int kk[ILP], jj[ILP], dk[ILP];
            walk_fetch<NT, ILP, TOMB>(G, sm, cnt, total, e0, per, g, j, kk, jj);
            gather_dist<ILP>(dr, kk, dk);
#pragma unroll
            for (int u = 0; u < ILP; ++u)
                if (kk[u] >= 0) edge(jj[u], sm.x[jj[u]], kk[u], dk[u]);
        }
        __syncthreads();
        if (t < cnt) post(t, sm.x[t]);
        __syncthreads();
    }
}

struct NoPost {
    __device__ void operator()(int, int) const {}
};

// Edge-balanced walk that sums one value per edge into the edge's source
// vertex: contrib(j, y, k, dist[k], v) returns whether edge (y,k) contributes
// and sets v.  Chunking, ILP and gathers are those of lb_walk (never counted as
// reference traversal).  Instead of one shared atomic per contributing edge,
// each thread keeps a running sum while its edges share a source vertex and
// flushes it into s_sum[j] (and ORs kSumHit into s_hit[j], which prep must
// initialise) only when the source changes; at the end of a chunk a warp whose
// lanes all hold the same source adds its sums with shuffles first.
// post(j, y) then sees the chunk's totals.
// GATHER = false skips the distance gather (contrib then receives 0), for
// walks whose edge test needs no distance.
constexpr int kSumHit = 4;
template <int NT, bool GATHER, int ILP = kEdgeIlp, bool TOMB = false, class Prep, class Contrib, class Post>
__device__ __forceinline__ void lb_walk_sum(const DevGraph& G, int g, const DistRow dr,
                                            const int32_t* l1, int n1, LbSmem<NT>& sm, double* s_sum, int* s_hit,
                                            Prep prep, Contrib contrib, Post post)
{
    for (int base = 0; base < n1; base += NT) {
        const int t = threadIdx.x;
        const int cnt = min(NT, n1 - base);
        int d = 0;
        if (t < cnt) {
            const int x = l1[base + t];
            const int64_t rs = G.row[x];
            d = vis_deg(G, x, rs, g);
            sm.x[t] = x;
            sm.row[t] = rs;
            s_sum[t] = 0.0;
            prep(t, x, d);
        }
        int total;
        const int off = block_exclusive_scan<NT>(d, sm.warp, &total);
        if (t < cnt) sm.off[t] = off;
        if (t == 0) {
            sm.off[cnt] = total;
            sm.scanned_e += (unsigned)total;
        }
        __syncthreads();
        int j = 0;
        int cj = -1;       // source vertex of the running sum
        double cs = 0.0;   // running sum
        const int per = min(ILP, (total + NT - 1) / NT);
        for (int e0 = t * per; e0 < total; e0 += NT * per) {
            int kk[ILP], jj[ILP], dk[ILP];
            walk_fetch<NT, ILP, TOMB>(G, sm, cnt, total, e0, per, g, j, kk, jj);
            if (GATHER) {
                gather_dist<ILP>(dr, kk, dk);
            } else {
#pragma unroll
                for (int u = 0; u < ILP; ++u) dk[u] = 0;
            }
#pragma unroll
            for (int u = 0; u < ILP; ++u) {
                double v;
                if (kk[u] >= 0 && contrib(jj[u], sm.x[jj[u]], kk[u], dk[u], v)) {
                    if (jj[u] != cj) {
                        if (cj >= 0) {
                            atomicAdd(&s_sum[cj], cs);
                            atomicOr(&s_hit[cj], kSumHit);
                        }
                        cj = jj[u];
                        cs = 0.0;
                    }
                    cs += v;
                }
            }
        }
        // The warp's largest running-sum source k0 (lanes without a sum
        // hold -1) is summed with shuffles and added once; lanes whose sum
        // belongs to another source add their own.  Sources are few and
        // consecutive lanes mostly share one (a hub's slots), and a shared
        // fp64 atomic per lane on the same address serialises.
        const unsigned full = 0xffffffffu;
        const int k0 = __reduce_max_sync(full, cj);
        if (k0 >= 0) {
            double v = cj == k0 ? cs : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(full, v, o);
            if ((t & 31) == 0) {
                atomicAdd(&s_sum[k0], v);
                atomicOr(&s_hit[k0], kSumHit);
            }
        }
        if (cj >= 0 && cj != k0) {
            atomicAdd(&s_sum[cj], cs);
            atomicOr(&s_hit[cj], kSumHit);
        }
        __syncthreads();
        if (t < cnt) post(t, sm.x[t]);
        __syncthreads();
    }
}

// Block-wide sums of two 64-bit integers and one double per thread; every
// thread gets the three totals.  Warps reduce with shuffles, then warp 0 adds
// the per-warp partials and publishes the totals.  GB300 issues fp64 at a
// small fraction of its fp32 rate (every warp-wide fp64 instruction holds the
// SM's fp64 pipe for many cycles), so the double is shuffled only in warps
// where some lane holds a nonzero value, and the tail is one warp's work
// rather than every thread adding all partials.  s_part holds 3 * (NT/32) + 3
// entries.
template <int NT>
__device__ __forceinline__ void block_sum3(long long& a, long long& b, double& c, long long* s_part)
{
    constexpr int NW = NT / 32;
    static_assert(NW <= 32, "one warp adds the partials");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(full, a, o);
        b += __shfl_xor_sync(full, b, o);
    }
    if (__any_sync(full, __double_as_longlong(c) != 0)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(full, c, o);
    }
    if (lane == 0) {
        s_part[3 * wid] = a;
        s_part[3 * wid + 1] = b;
        s_part[3 * wid + 2] = __double_as_longlong(c);
    }
    __syncthreads();
    if (wid == 0) {
        long long xa = 0, xb = 0, xc = 0;
        if (lane < NW) {
            xa = s_part[3 * lane];
            xb = s_part[3 * lane + 1];
            xc = s_part[3 * lane + 2];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            xa += __shfl_xor_sync(full, xa, o);
            xb += __shfl_xor_sync(full, xb, o);
        }
        double dc = __longlong_as_double(xc);
        if (__any_sync(full, xc != 0)) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) dc += __shfl_xor_sync(full, dc, o);
        }
        if (lane == 0) {
            s_part[3 * NW] = xa;
            s_part[3 * NW + 1] = xb;
            s_part[3 * NW + 2] = __double_as_longlong(dc);
        }
    }
    __syncthreads();
    a = s_part[3 * NW];
    b = s_part[3 * NW + 1];
    c = __longlong_as_double(s_part[3 * NW + 2]);
    __syncthreads();
}

// Block-wide sum of one 64-bit value per thread (all threads get the total);
// same scheme and s_part size as block_sum3.
template <int NT>
__device__ __forceinline__ long long block_sum(long long v, long long* s_part)
{
    constexpr int NW = NT / 32;
    static_assert(NW <= 32, "one warp adds the partials");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(full, v, o);
    if (lane == 0) s_part[wid] = v;
    __syncthreads();
    if (wid == 0) {
        long long x = lane < NW ? s_part[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(full, x, o);
        if (lane == 0) s_part[3 * NW] = x;
    }
    __syncthreads();
    const long long t = s_part[3 * NW];
    __syncthreads();
    return t;
}

}  // namespace sbc
