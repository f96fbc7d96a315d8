// Whole-GPU recompute of a few roots' trees (for deletions).
//
// A deletion that leaves the deeper endpoint without a parent has its root
// recomputed from scratch (the state of the modified graph, by definition).
// The static kernel gives each root one CTA, which suits many roots at once;
// a deletion on a large graph recomputes only a few, and one CTA walking a
// 10^6-vertex graph takes ~100 ms.  Here those roots are recomputed together
// by the whole GPU, level-synchronously (BrandesSingleTree,
// src/streamingbc_init.c:87-183), every level one launch for all of them
// (blockIdx.y = the root's slot):
//   k_rows_reset     each root's dist / dist8 / sigma / delta row to "unreached"
//   k_wide_forward   warp per frontier vertex, lanes over its adjacency: an
//                    unreached neighbour is claimed for the next level by CAS on
//                    its distance and appended to the BFS order; every
//                    neighbour on the next level gains the vertex's sigma (int64
//                    atomics, exact)
//   k_wide_backward  warp per vertex of a level, deepest first: its children's
//                    w = (delta+1)/sigma summed with shuffles; delta and w set
// Slot j's BFS order and w live in worker j's scratch (no update job runs at
// the same time: deletions are applied between batches on the graph's stream);
// w is cleared afterwards.
#include <vector>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

// Roots recomputed together: slot j (blockIdx.y) recomputes root rows[j] in
// worker j's scratch (its qd slice holds the BFS order, its acc slice w).
struct WideArgs {
    int32_t* dist;
    uint8_t* dist8;
    int64_t* sigma;
    double* delta;
    const int64_t* roots;
    const int* rows;
    int64_t nv;
    int32_t* qd;                // worker-major, nv per worker
    double* acc;                // worker-major, nv per worker
    int* count;                 // [slots] BFS order length of each slot
    const int2* range;          // [slots] (start, length) of the level being walked
    unsigned long long* counters;
};

__global__ void k_rows_reset(const WideArgs A)
{
    const int j = blockIdx.y;
    const int r = A.rows[j];
    const size_t o = (size_t)r * A.nv;
    const int64_t root = A.roots[r];
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < A.nv; x += (int64_t)gridDim.x * blockDim.x) {
        const bool is_root = x == root;
        A.dist[o + x] = is_root ? 0 : SBC_INF;
        A.dist8[o + x] = is_root ? 0 : SBC_D8_INF;
        A.sigma[o + x] = is_root ? 1 : 0;
        A.delta[o + x] = 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.qd[(size_t)j * A.nv] = (int32_t)root;
        A.count[j] = 1;
    }
}

__global__ void k_wide_forward(DevGraph G, const WideArgs A, int L)
{
    const int j = blockIdx.y;
    const int2 rg = A.range[j];
    if (rg.y == 0) return;
    const size_t o = (size_t)A.rows[j] * A.nv;
    int32_t* D = A.dist + o;
    uint8_t* D8 = A.dist8 + o;
    int64_t* S = A.sigma + o;
    int32_t* order = A.qd + (size_t)j * A.nv;
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); i < rg.y; i += nwarps) {
        const int x = order[rg.x + i];
        const int64_t rx = G.row[x];
        const int dx = G.deg[x];
        const int64_t sx = S[x];
        for (int s = lane; s < dx; s += 32) {
            const int k = G.col[rx + s];
            const int old = atomicCAS(&D[k], SBC_INF, L + 1);
            if (old == SBC_INF) {
                D8[k] = enc_d8(L + 1);
                order[atomicAdd(&A.count[j], 1)] = k;
            }
            if (old == SBC_INF || old == L + 1) atomic_add_i64(&S[k], sx);
        }
        if (lane == 0) {
            atomicAdd(&A.counters[0], 1ull);
            atomicAdd(&A.counters[1], (unsigned long long)dx);
        }
    }
}

__global__ void k_wide_backward(DevGraph G, const WideArgs A, int L)
{
    const int j = blockIdx.y;
    const int2 rg = A.range[j];
    if (rg.y == 0) return;
    const size_t o = (size_t)A.rows[j] * A.nv;
    const int32_t* D = A.dist + o;
    const int64_t* S = A.sigma + o;
    double* Dl = A.delta + o;
    double* w = A.acc + (size_t)j * A.nv;
    const int32_t* lvl = A.qd + (size_t)j * A.nv + rg.x;
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); i < rg.y; i += nwarps) {
        const int x = lvl[i];
        const int64_t rx = G.row[x];
        const int dx = G.deg[x];
        double sum = 0.0;
        for (int s = lane; s < dx; s += 32) {
            const int k = G.col[rx + s];
            if (D[k] == L + 1) sum += w[k];
        }
        if (__any_sync(0xffffffffu, sum != 0.0)) {
#pragma unroll
            for (int o2 = 16; o2 > 0; o2 >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o2);
        }
        if (lane == 0) {
            const double sx = (double)S[x];
            const double d = sx * sum;
            Dl[x] = d;
            w[x] = (d + 1.0) / sx;
            atomicAdd(&A.counters[0], 1ull);
            atomicAdd(&A.counters[1], (unsigned long long)dx);
        }
    }
}

__global__ void k_clear_w(const WideArgs A)
{
    const int j = blockIdx.y;
    const int32_t* order = A.qd + (size_t)j * A.nv;
    double* w = A.acc + (size_t)j * A.nv;
    const int n = A.count[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w[order[i]] = 0.0;
}

// Recomputes the listed root rows of forest f (d_rows: the same list on the
// device), as many at a time as the forest has workers; synchronous (one
// device-to-host read of every slot's BFS length per level).
cudaError_t recompute_roots_wide(sbc_forest* f, const std::vector<int>& rows, const int* d_rows)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    const int64_t nv = f->nv;
    const DevGraph G = g->dev();
    cudaError_t e;
    if (!f->d_wide) {
        // per slot: BFS length, then the (start, length) range of the level walked
        if ((e = cudaMalloc(&f->d_wide, sizeof(int) * 3 * kWideRecompute))) return e;
    }
    WideArgs A;
    A.dist = f->d_dist;
    A.dist8 = f->d_dist8;
    A.sigma = f->d_sigma;
    A.delta = f->d_delta;
    A.roots = f->d_roots;
    A.nv = nv;
    A.qd = f->ws.qd;
    A.acc = f->ws.acc;
    A.count = f->d_wide;
    A.range = reinterpret_cast<const int2*>(f->d_wide + kWideRecompute);
    A.counters = f->d_counters;
    int2* d_range = reinterpret_cast<int2*>(f->d_wide + kWideRecompute);
    const int per = (int)std::min<int64_t>(std::min<int64_t>(f->workers, kWideRecompute), (int64_t)rows.size());
    for (size_t base = 0; base < rows.size(); base += (size_t)per) {
        const int nr = (int)std::min<size_t>((size_t)per, rows.size() - base);
        A.rows = d_rows + base;
        const int gx = std::max(1, f->sm_count * 8 / nr);
        k_rows_reset<<<dim3(gx, nr), 256, 0, s>>>(A);
        // forward: levels of every slot at once
        std::vector<std::vector<int>> off(nr, std::vector<int>{0, 1});
        std::vector<int2> rg(nr);
        std::vector<int> cnt(nr);
        for (int L = 0;; ++L) {
            bool any = false;
            for (int j = 0; j < nr; ++j) {
                const int lo = off[j][L], hi = off[j][L + 1];
                rg[j] = make_int2(lo, hi - lo);
                any |= hi > lo;
            }
            if (!any) break;
            if ((e = cudaMemcpyAsync(d_range, rg.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice, s))) return e;
            k_wide_forward<<<dim3(gx, nr), 256, 0, s>>>(G, A, L);
            if ((e = cudaMemcpyAsync(cnt.data(), A.count, sizeof(int) * nr, cudaMemcpyDeviceToHost, s)) ||
                (e = cudaStreamSynchronize(s)))
                return e;
            for (int j = 0; j < nr; ++j) off[j].push_back(cnt[j]);
        }
        // backward: deepest level first; a slot's levels 0 .. off.size()-3 are non-empty
        size_t maxl = 0;
        for (int j = 0; j < nr; ++j) maxl = std::max(maxl, off[j].size());
        for (int L = (int)maxl - 3; L >= 0; --L) {
            for (int j = 0; j < nr; ++j) {
                const bool has = L + 1 < (int)off[j].size() - 1;
                rg[j] = has ? make_int2(off[j][L], off[j][L + 1] - off[j][L]) : make_int2(0, 0);
            }
            if ((e = cudaMemcpyAsync(d_range, rg.data(), sizeof(int2) * nr, cudaMemcpyHostToDevice, s))) return e;
            k_wide_backward<<<dim3(gx, nr), 256, 0, s>>>(G, A, L);
        }
        k_clear_w<<<dim3(gx, nr), 256, 0, s>>>(A);
        if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(s))) return e;  // range / count reused next group
    }
    return cudaSuccess;
}

}  // namespace sbc
