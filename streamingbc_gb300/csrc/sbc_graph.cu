// Device slack-CSR adjacency: in-place insertion and re-pack.
//
// Replaces stinger_insert_edge (src/stinger/stinger.c:778-876) and the edge
// block pool.  Each vertex owns slots [row[v], row[v]+cap[v]); the first deg[v]
// hold live neighbours.  An insertion appends into the slack of both endpoints
// (one direction for the directed form) after a duplicate check, and stamps the
// slot with the insertion's index inside its batch (seq), so that a traversal
// for insertion i of a batch sees only edges of insertions <= i.
#include <climits>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

// Insertion outcome codes written to ok[i]:
//   1 inserted, 0 duplicate (edge already present), -1 self loop or id out of
//   range, -2 no slack left (the host plans capacity so this is not expected).
__device__ __forceinline__ void append_warp(int64_t nv, const int64_t* __restrict__ row, int32_t* deg,
                                            const int32_t* __restrict__ cap, int32_t* col, int32_t* seq, int n,
                                            const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                                            int32_t* ok, int directed, int* err)
{
    const int lane = threadIdx.x;
    for (int i = 0; i < n; ++i) {
        const int u = iu[i], v = iv[i];
        int code = 1;
        if (u == v || u < 0 || v < 0 || u >= nv || v >= nv) code = -1;
        if (code == 1) {
            int x = u, y = v;
            if (!directed && deg[v] < deg[u]) {
                x = v;
                y = u;
            }
            const int dx = deg[x];
            const int64_t rx = row[x];
            bool found = false;
            for (int s = lane; s < dx; s += 32)
                if (col[rx + s] == y) found = true;
            if (__any_sync(0xffffffffu, found)) code = 0;
        }
        if (code == 1 && !(deg[u] < cap[u] && (directed || deg[v] < cap[v]))) {
            code = -2;
            if (lane == 0) atomicOr(err, 1);
        }
        if (lane == 0) {
            if (code == 1) {
                int p = deg[u];
                col[row[u] + p] = v;
                seq[row[u] + p] = i;
                deg[u] = p + 1;
                if (!directed) {
                    p = deg[v];
                    col[row[v] + p] = u;
                    seq[row[v] + p] = i;
                    deg[v] = p + 1;
                }
            }
            ok[i] = code;
        }
        __syncwarp();
    }
}

__global__ void k_append(int64_t nv, const int64_t* __restrict__ row, int32_t* deg, const int32_t* __restrict__ cap,
                         int32_t* col, int32_t* seq, int n, const int32_t* __restrict__ iu,
                         const int32_t* __restrict__ iv, int32_t* ok, int directed, int* err)
{
    append_warp(nv, row, deg, cap, col, seq, n, iu, iv, ok, directed, err);
}

// The same results with a warp per insertion, in three launches:
//   k_append_codes  -1 bad id or loop; 0 an edge already (of the graph as the
//                   batch begins -- sealed, so a binary search of the sorted
//                   slots plus a scan of any tail -- or of an earlier
//                   insertion of the batch); 1 to insert.
//   k_append_rank   each insertion's rank among the batch's insertions at
//                   each endpoint (its slot past deg0, so that every vertex's
//                   appended slots stay in insertion order), and whether
//                   every slot fits the vertex's slack.
//   k_append_place  the slots written (seq = index) and the degrees raised;
//                   if some slot does not fit, one warp appends the whole
//                   batch in order instead (k_append's way), so that exactly
//                   the insertions a one-by-one append rejects are rejected.
// rk holds 2 n ranks and, at rk[2 n], the misfit flag.
__global__ void k_append_codes(int64_t nv, const int64_t* __restrict__ row, const int32_t* __restrict__ deg,
                               const int32_t* __restrict__ nsort, const int32_t* __restrict__ col, int n,
                               const int32_t* __restrict__ iu, const int32_t* __restrict__ iv, int32_t* ok,
                               int directed, int32_t* rk)
{
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w == 0 && lane == 0) rk[2 * n] = 0;
    if (w >= n) return;
    const int u = iu[w], v = iv[w];
    int code = (u == v || u < 0 || v < 0 || u >= nv || v >= nv) ? -1 : 1;
    if (code == 1) {
        bool dup = false;
        for (int base = 0; base < w && !dup; base += 32) {
            const int j = base + lane;
            bool same = false;
            if (j < w) {
                const int a = iu[j], b = iv[j];
                same = (a == u && b == v) || (!directed && a == v && b == u);
            }
            dup = __any_sync(0xffffffffu, same);
        }
        if (dup) code = 0;
    }
    if (code == 1) {
        int x = u, y = v;
        if (!directed && deg[v] < deg[u]) {
            x = v;
            y = u;
        }
        const int64_t rx = row[x];
        const int d = deg[x], ns = min(nsort[x], d);
        bool found = false;
        if (lane == 0) {
            int lo = 0, hi = ns;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const int c = col[rx + mid];
                if (c < y) lo = mid + 1;
                else if (c > y) hi = mid;
                else {
                    found = true;
                    break;
                }
            }
        }
        for (int s = ns + lane; s < d; s += 32)
            if (col[rx + s] == y) found = true;
        if (__any_sync(0xffffffffu, found)) code = 0;
    }
    if (lane == 0) ok[w] = code;
}

__global__ void k_append_rank(const int32_t* __restrict__ deg0, const int32_t* __restrict__ cap, int n,
                              const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                              const int32_t* __restrict__ ok, int directed, int32_t* rk)
{
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n || ok[w] != 1) return;
    const int u = iu[w], v = iv[w];
    int ru = 0, rv = 0;
    for (int j = lane; j < w; j += 32) {
        if (ok[j] != 1) continue;
        const int a = iu[j], b = iv[j];
        ru += (a == u || (!directed && b == u)) ? 1 : 0;
        rv += (a == v || b == v) ? 1 : 0;
    }
    ru = __reduce_add_sync(0xffffffffu, ru);
    rv = __reduce_add_sync(0xffffffffu, rv);
    if (lane == 0) {
        rk[w] = ru;
        rk[n + w] = rv;
        if (deg0[u] + ru >= cap[u] || (!directed && deg0[v] + rv >= cap[v])) atomicOr(&rk[2 * n], 1);
    }
}

__global__ void k_append_place(int64_t nv, const int64_t* __restrict__ row, int32_t* deg,
                               const int32_t* __restrict__ deg0, const int32_t* __restrict__ cap, int32_t* col,
                               int32_t* seq, int n, const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                               int32_t* ok, int directed, const int32_t* __restrict__ rk, int* err)
{
    if (rk[2 * n]) {
        // a slot does not fit: the whole batch in order, one warp
        if (blockIdx.x == 0 && threadIdx.x < 32)
            append_warp(nv, row, deg, cap, col, seq, n, iu, iv, ok, directed, err);
        return;
    }
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || ok[i] != 1) return;
    const int u = iu[i], v = iv[i];
    const int pu = deg0[u] + rk[i];
    col[row[u] + pu] = v;
    seq[row[u] + pu] = i;
    atomicMax(&deg[u], pu + 1);
    if (!directed) {
        const int pv = deg0[v] + rk[n + i];
        col[row[v] + pv] = u;
        seq[row[v] + pv] = i;
        atomicMax(&deg[v], pv + 1);
    }
}

// Many graphs' batches at once: one warp (CTA) per graph, each appending its
// graph's insertions in order exactly as k_append does.
__global__ void k_append_group(const __grid_constant__ GraphBatchSlots S)
{
    const GraphBatchSlot& b = S.slot[blockIdx.x];
    append_warp(b.nv, b.row, b.deg, b.cap, b.col, b.seq, b.n, b.iu, b.iv, b.ok, 0, b.err);
}

// A batch's endpoint arrays live in the caller's device memory.  k_set_src
// records their addresses in the graph's two-pointer slot (its arguments are
// copied at launch, so nothing on the host has to outlive the call), and
// k_stage_inputs, which a captured batch graph replays unchanged, copies from
// the addresses in the slot into the staging rows (u at dst[0..n), v at
// dst[cap..cap+n)).
__global__ void k_set_src(const int32_t** slot, const int32_t* u, const int32_t* v)
{
    slot[0] = u;
    slot[1] = v;
}

__global__ void k_stage_inputs(const int32_t* const* __restrict__ slot, int32_t* dst, int cap, int n)
{
    const int32_t* u = slot[0];
    const int32_t* v = slot[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dst[i] = u[i];
        dst[cap + i] = v[i];
    }
}

cudaError_t launch_set_src(sbc_graph* g, const int32_t* d_u, const int32_t* d_v)
{
    k_set_src<<<1, 1, 0, g->stream>>>(g->d_src, d_u, d_v);
    return cudaGetLastError();
}

cudaError_t launch_stage(sbc_graph* g, int n)
{
    const int blocks = std::min((n + 255) / 256, 1024);
    k_stage_inputs<<<blocks < 1 ? 1 : blocks, 256, 0, g->stream>>>(g->d_src, g->d_ins, g->ins_capacity, n);
    return cudaGetLastError();
}

// After a batch's update: the slots it appended to a vertex (an unsorted tail
// after the first nsort[x] slots, which are sorted by neighbour id) are merged
// into the sorted prefix, so that edge tests (has_edge: binary search of the
// prefix, then a scan of the tail) never scan more than the current batch's
// appends -- without this a hub's tail grew by every insertion on it.  One
// block per endpoint of an applied insertion; the first block to reach a
// vertex claims it by swapping its deg0 for -1 (the seal that follows rewrites
// deg0 = deg for the same endpoints; the update that read deg0 has finished).
// The tail (at most kMergeTail slots per batch; a longer one is merged over
// several batches) is sorted in shared memory; each tail value's final slot is
// its rank among the tail plus its lower bound in the prefix; prefix values
// move up by the number of tail values below them, in chunks from the end, so
// no value is overwritten before it is read.  seq of the moved slots is not
// read again (after the seal every slot is below deg0).
constexpr int kMergeTail = 2048;
constexpr int kMergeThreads = 256;
constexpr int kMergeRun = 8;  // prefix values per thread per chunk

__device__ __forceinline__ void merge_tail(const int64_t* __restrict__ row, const int32_t* __restrict__ deg,
                                           int32_t* deg0, int32_t* nsort, int32_t* col, int x)
{
    __shared__ int s_tail[kMergeTail];
    __shared__ int s_dst[kMergeTail];
    __shared__ int s_claim;
    const int tid = threadIdx.x;
    if (tid == 0) s_claim = atomicExch(&deg0[x], -1);
    __syncthreads();
    if (s_claim < 0) return;  // another block merges x
    const int ns = nsort[x];
    const int t = min(deg[x] - ns, kMergeTail);
    if (t <= 0) return;
    const int64_t rx = row[x];
    int P = 1;
    while (P < t) P <<= 1;
    for (int k = tid; k < P; k += kMergeThreads) s_tail[k] = k < t ? col[rx + ns + k] : INT_MAX;
    __syncthreads();
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = tid; i < (P >> 1); i += kMergeThreads) {
                const int lo = (i / stride) * 2 * stride + (i % stride);
                const int hi = lo + stride;
                const int a = s_tail[lo], b = s_tail[hi];
                if ((a > b) == ((lo & size) == 0)) {
                    s_tail[lo] = b;
                    s_tail[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    for (int k = tid; k < t; k += kMergeThreads) {
        const int v = s_tail[k];
        int lo = 0, hi = ns;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (col[rx + mid] < v) lo = mid + 1;
            else hi = mid;
        }
        s_dst[k] = lo + k;
    }
    __syncthreads();
    const int first = s_dst[0];  // prefix values below it stay where they are
    constexpr int kChunk = kMergeThreads * kMergeRun;
    for (int c1 = ns; c1 > first; c1 -= kChunk) {
        const int c0 = max(first, c1 - kChunk);
        int val[kMergeRun], dst[kMergeRun];
#pragma unroll
        for (int r = 0; r < kMergeRun; ++r) {
            const int idx = c0 + tid + r * kMergeThreads;
            dst[r] = -1;
            if (idx < c1) {
                const int v = col[rx + idx];
                int lo = 0, hi = t;  // tail values below v
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (s_tail[mid] < v) lo = mid + 1;
                    else hi = mid;
                }
                val[r] = v;
                dst[r] = idx + lo;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kMergeRun; ++r)
            if (dst[r] >= 0) col[rx + dst[r]] = val[r];
        __syncthreads();
    }
    for (int k = tid; k < t; k += kMergeThreads) col[rx + s_dst[k]] = s_tail[k];
    if (tid == 0) nsort[x] = ns + t;
}

__global__ void __launch_bounds__(kMergeThreads) k_merge_tails(int n, const int32_t* __restrict__ iu,
                                                               const int32_t* __restrict__ iv,
                                                               const int32_t* __restrict__ ok,
                                                               const int64_t* __restrict__ row,
                                                               const int32_t* __restrict__ deg, int32_t* deg0,
                                                               int32_t* nsort, int32_t* col)
{
    const int e = blockIdx.x;
    const int i = e < n ? e : e - n;
    if (ok[i] <= 0) return;
    merge_tail(row, deg, deg0, nsort, col, e < n ? iu[i] : iv[i]);
}

// k_merge_tails over many graphs: blockIdx.y selects the graph.
__global__ void __launch_bounds__(kMergeThreads) k_merge_tails_group(const __grid_constant__ GraphBatchSlots S)
{
    const GraphBatchSlot& b = S.slot[blockIdx.y];
    const int e = blockIdx.x;
    if (e >= 2 * b.n) return;
    const int i = e < b.n ? e : e - b.n;
    if (b.ok[i] <= 0) return;
    merge_tail(b.row, b.deg, b.deg0, b.nsort, b.col, e < b.n ? b.iu[i] : b.iv[i]);
}

// After a batch: every appended slot becomes visible to all later traversals.
__global__ void k_seal(int n, const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                       const int32_t* __restrict__ ok, const int32_t* __restrict__ deg, int32_t* deg0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || ok[i] <= 0) return;
    deg0[iu[i]] = deg[iu[i]];
    deg0[iv[i]] = deg[iv[i]];
}

// Removes neighbour y from x's slots (one warp): the slot is found, the later
// slots move down one place (a sorted prefix stays sorted), and deg -- and
// deg0 / nsort when the slot lay below them -- drop by one.  Returns whether y
// was present.
__device__ __forceinline__ bool remove_slot(const int64_t* __restrict__ row, int32_t* deg, int32_t* deg0,
                                            int32_t* nsort, int32_t* col, int32_t* seq, int x, int y)
{
    const int lane = threadIdx.x & 31;
    const int d = deg[x];
    const int64_t rx = row[x];
    int p = -1;
    for (int base = 0; base < d && p < 0; base += 32) {
        const int s = base + lane;
        const unsigned m = __ballot_sync(0xffffffffu, s < d && col[rx + s] == y);
        if (m) p = base + __ffs(m) - 1;
    }
    if (p < 0) return false;
    for (int base = p; base < d - 1; base += 32) {
        const int s = base + lane;
        int c = 0, q = 0;
        if (s < d - 1) {
            c = col[rx + s + 1];
            q = seq[rx + s + 1];
        }
        __syncwarp();  // every lane has read before any slot is overwritten
        if (s < d - 1) {
            col[rx + s] = c;
            seq[rx + s] = q;
        }
        __syncwarp();
    }
    if (lane == 0) {
        deg[x] = d - 1;
        if (p < deg0[x]) deg0[x] -= 1;
        if (p < nsort[x]) nsort[x] -= 1;
    }
    __syncwarp();
    return true;
}

// Edge removal (stinger_remove_edge, src/stinger/stinger.c): (u,v) and,
// unless directed, (v,u); *res = 1 removed, 0 absent, -1 self loop or id out
// of range.  One warp; the graph's stream orders it with the batches.
__global__ void k_remove(int64_t nv, const int64_t* __restrict__ row, int32_t* deg, int32_t* deg0, int32_t* nsort,
                         int32_t* col, int32_t* seq, int u, int v, int directed, int* res)
{
    int code;
    if (u == v || u < 0 || v < 0 || u >= nv || v >= nv) {
        code = -1;
    } else {
        code = remove_slot(row, deg, deg0, nsort, col, seq, u, v) ? 1 : 0;
        if (!directed) remove_slot(row, deg, deg0, nsort, col, seq, v, u);
    }
    if (threadIdx.x == 0) *res = code;
}

// Batched deletions, step 1: the n staged edges (iu/iv, -1 = invalid id) are
// removed in order, each only marked -- its two slots keep their place and get
// seq = -1 - i -- so that every deletion's update can still see the graph as
// it stood before it (a slot removed at deletion j is an edge for jobs i < j).
// code[i] = 1 removed, 0 absent (never there, or removed earlier in the
// batch), -1 self loop / bad id.  One thread: each lookup is a binary search
// of the sorted leading slots, then a scan of any unsorted tail.
__device__ __forceinline__ int64_t live_slot(const int64_t* row, const int32_t* deg, const int32_t* nsort,
                                             const int32_t* col, const int32_t* seq, int x, int y)
{
    const int64_t rx = row[x];
    const int d = deg[x], ns = min(nsort[x], d);
    int lo = 0, hi = ns;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col[rx + mid];
        if (c < y) lo = mid + 1;
        else if (c > y) hi = mid;
        else return seq[rx + mid] >= 0 ? rx + mid : -1;
    }
    for (int s2 = ns; s2 < d; ++s2)
        if (col[rx + s2] == y && seq[rx + s2] >= 0) return rx + s2;
    return -1;
}

__global__ void k_mark_removed(const int64_t* __restrict__ row, const int32_t* __restrict__ deg,
                               const int32_t* __restrict__ nsort, const int32_t* __restrict__ col, int32_t* seq, int n,
                               const int32_t* __restrict__ iu, const int32_t* __restrict__ iv, int32_t* code)
{
    if (threadIdx.x != 0) return;
    for (int i = 0; i < n; ++i) {
        const int u = iu[i], v = iv[i];
        if (u < 0 || v < 0 || u == v) {
            code[i] = -1;
            continue;
        }
        const int64_t pu = live_slot(row, deg, nsort, col, seq, u, v);
        const int64_t pv = pu < 0 ? -1 : live_slot(row, deg, nsort, col, seq, v, u);
        if (pu < 0 || pv < 0) {
            code[i] = 0;
            continue;
        }
        seq[pu] = -1 - i;
        seq[pv] = -1 - i;
        code[i] = 1;
    }
}

// Batched deletions, step 3 (after the update): the marked slots leave their
// lists, which keep their order.  CTA per deletion endpoint; the first CTA to
// reach a vertex claims it by swapping its deg0 (== deg between batches) for
// -1 until it is done, and CTAs that find it claimed leave it (one arriving
// after the claimer finished compacts a clean list again, which changes
// nothing).
__global__ void __launch_bounds__(256) k_compact_removed(const int64_t* __restrict__ row, int32_t* deg, int32_t* deg0,
                                                         int32_t* nsort, int32_t* col, int32_t* seq, int n,
                                                         const int32_t* __restrict__ iu,
                                                         const int32_t* __restrict__ iv,
                                                         const int32_t* __restrict__ code)
{
    __shared__ int s_warp[8];
    __shared__ int s_keep_sorted;
    __shared__ int s_mine;
    const int i = blockIdx.x >> 1;
    if (code[i] != 1) return;
    const int x = (blockIdx.x & 1) ? iv[i] : iu[i];
    if (threadIdx.x == 0) {
        const int d0 = deg0[x];
        s_mine = d0 >= 0 && atomicCAS(&deg0[x], d0, -1) == d0;
    }
    __syncthreads();
    if (!s_mine) return;
    const int64_t rx = row[x];
    const int d = deg[x], ns = min(nsort[x], d);
    if (threadIdx.x == 0) s_keep_sorted = 0;
    int kept = 0;
    for (int base = 0; base < d; base += 256) {
        const int sl = base + (int)threadIdx.x;
        int c = 0, q = 0;
        bool keep = false;
        if (sl < d) {
            c = col[rx + sl];
            q = seq[rx + sl];
            keep = q >= 0;
        }
        int total;
        const int off = block_exclusive_scan<256>(keep ? 1 : 0, s_warp, &total);  // every read precedes its barrier
        if (keep) {
            col[rx + kept + off] = c;
            seq[rx + kept + off] = q;
        }
        if (keep && sl < ns) atomicAdd(&s_keep_sorted, 1);
        kept += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        deg[x] = kept;
        deg0[x] = kept;
        nsort[x] = s_keep_sorted;
    }
}

// k_seal over many graphs: blockIdx.y selects the graph.
__global__ void k_seal_group(const __grid_constant__ GraphBatchSlots S)
{
    const GraphBatchSlot& b = S.slot[blockIdx.y];
    if (S.errs && blockIdx.x == 0 && threadIdx.x == 0) S.errs[blockIdx.y] = *b.err;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.n || b.ok[i] <= 0) return;
    b.deg0[b.iu[i]] = b.deg[b.iu[i]];
    b.deg0[b.iv[i]] = b.deg[b.iv[i]];
}

// Copy every vertex's live slots to a new layout with larger slack (warp per vertex).
__global__ void k_repack(int64_t nv, const int64_t* __restrict__ orow, const int32_t* __restrict__ deg,
                         const int32_t* __restrict__ ocol, const int32_t* __restrict__ oseq,
                         const int64_t* __restrict__ nrow, int32_t* __restrict__ ncol, int32_t* __restrict__ nseq)
{
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nv; v += nwarps) {
        const int d = deg[v];
        const int64_t a = orow[v], b = nrow[v];
        for (int s = lane; s < d; s += 32) {
            ncol[b + s] = ocol[a + s];
            nseq[b + s] = oseq[a + s];
        }
    }
}

cudaError_t launch_append(sbc_graph* g, int n, bool directed)
{
    const int32_t* iu = g->d_ins;
    const int32_t* iv = g->d_ins + g->ins_capacity;
    int32_t* ok = g->d_ins + 2 * g->ins_capacity;
    g->last_directed = directed;
    if (n <= 0) return cudaSuccess;
    if (n > kParallelAppendMax) {
        // the parallel form's within-batch tests grow with n^2
        k_append<<<1, 32, 0, g->stream>>>(g->nv, g->d_row, g->d_deg, g->d_cap, g->d_col, g->d_seq, n, iu, iv, ok,
                                          directed ? 1 : 0, g->d_err);
        return cudaGetLastError();
    }
    int32_t* rk = g->d_ins + 3 * g->ins_capacity;
    const int wblocks = (n + 7) / 8;  // 8 warps of 32 per block, a warp per insertion
    k_append_codes<<<wblocks, 256, 0, g->stream>>>(g->nv, g->d_row, g->d_deg, g->d_nsort, g->d_col, n, iu, iv, ok,
                                                   directed ? 1 : 0, rk);
    k_append_rank<<<wblocks, 256, 0, g->stream>>>(g->d_deg0, g->d_cap, n, iu, iv, ok, directed ? 1 : 0, rk);
    k_append_place<<<(n + 255) / 256, 256, 0, g->stream>>>(g->nv, g->d_row, g->d_deg, g->d_deg0, g->d_cap, g->d_col,
                                                           g->d_seq, n, iu, iv, ok, directed ? 1 : 0, rk, g->d_err);
    return cudaGetLastError();
}

cudaError_t launch_seal(sbc_graph* g, int n)
{
    const int32_t* iu = g->d_ins;
    const int32_t* iv = g->d_ins + g->ins_capacity;
    const int32_t* ok = g->d_ins + 2 * g->ins_capacity;
    if (n <= 0) return cudaSuccess;
    k_merge_tails<<<2 * n, kMergeThreads, 0, g->stream>>>(n, iu, iv, ok, g->d_row, g->d_deg, g->d_deg0, g->d_nsort,
                                                          g->d_col);
    k_seal<<<(n + 255) / 256, 256, 0, g->stream>>>(n, iu, iv, ok, g->d_deg, g->d_deg0);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    return launch_l2mask_insert(g, n, g->last_directed);
}

GraphBatchSlot graph_batch_slot(sbc_graph* g, int n)
{
    GraphBatchSlot b;
    b.nv = g->nv;
    b.row = g->d_row;
    b.deg = g->d_deg;
    b.deg0 = g->d_deg0;
    b.nsort = g->d_nsort;
    b.cap = g->d_cap;
    b.col = g->d_col;
    b.seq = g->d_seq;
    b.iu = g->d_ins;
    b.iv = g->d_ins + g->ins_capacity;
    b.ok = g->d_ins + 2 * g->ins_capacity;
    b.err = g->d_err;
    b.n = n;
    return b;
}

cudaError_t launch_append_group(const GraphBatchSlots& S, cudaStream_t s)
{
    if (S.count <= 0) return cudaSuccess;
    k_append_group<<<S.count, 32, 0, s>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_seal_group(const GraphBatchSlots& S, cudaStream_t s)
{
    int nmax = 0;
    for (int i = 0; i < S.count; ++i) nmax = std::max(nmax, S.slot[i].n);
    if (S.count <= 0 || nmax <= 0) return cudaSuccess;
    k_merge_tails_group<<<dim3(2 * nmax, S.count), kMergeThreads, 0, s>>>(S);
    k_seal_group<<<dim3((nmax + 255) / 256, S.count), 256, 0, s>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_remove(sbc_graph* g, int u, int v, bool directed, int* d_res)
{
    k_remove<<<1, 32, 0, g->stream>>>(g->nv, g->d_row, g->d_deg, g->d_deg0, g->d_nsort, g->d_col, g->d_seq, u, v,
                                      directed ? 1 : 0, d_res);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    return launch_l2mask_remove(g, u, v, directed, d_res);
}

cudaError_t launch_mark_removed(sbc_graph* g, int n)
{
    k_mark_removed<<<1, 32, 0, g->stream>>>(g->d_row, g->d_deg, g->d_nsort, g->d_col, g->d_seq, n, g->d_ins,
                                           g->d_ins + g->ins_capacity, g->d_ins + 2 * g->ins_capacity);
    return cudaGetLastError();
}

cudaError_t launch_compact_removed(sbc_graph* g, int n)
{
    if (n <= 0) return cudaSuccess;
    k_compact_removed<<<2 * n, 256, 0, g->stream>>>(g->d_row, g->d_deg, g->d_deg0, g->d_nsort, g->d_col, g->d_seq, n,
                                                    g->d_ins, g->d_ins + g->ins_capacity,
                                                    g->d_ins + 2 * g->ins_capacity);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    return launch_l2mask_remove_batch(g, n);
}

cudaError_t launch_repack(sbc_graph* g, const int64_t* d_new_row, int32_t* d_new_col, int32_t* d_new_seq)
{
    int64_t blocks = (g->nv * 32 + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (blocks < 1) blocks = 1;
    k_repack<<<(int)blocks, 256, 0, g->stream>>>(g->nv, g->d_row, g->d_deg, g->d_col, g->d_seq, d_new_row, d_new_col,
                                                 d_new_seq);
    return cudaGetLastError();
}

}  // namespace sbc
