// Whole-GPU recompute of one root's tree (for deletions).
//
// A deletion that leaves the deeper endpoint without a parent has its root
// recomputed from scratch (the state of the modified graph, by definition).
// The static kernel gives each root one CTA, which suits many roots at once;
// a deletion on a large graph recomputes only a few, and one CTA walking a
// 10^6-vertex graph takes ~100 ms.  Here each root is recomputed by the whole
// GPU, level-synchronously (BrandesSingleTree, src/streamingbc_init.c:87-183,
// with every level a kernel launch):
//   k_row_reset      the root's dist / dist8 / sigma / delta row to "unreached"
//   k_wide_forward   warp per frontier vertex, lanes over its adjacency: an
//                    unreached neighbour is claimed for the next level by CAS on
//                    its distance and appended to the BFS order; every
//                    neighbour on the next level gains the vertex's sigma (int64
//                    atomics, exact)
//   k_wide_backward  warp per vertex of a level, deepest first: its children's
//                    w = (delta+1)/sigma summed with shuffles; delta and w set
// The BFS order and w live in worker 0's scratch (no update job runs at the
// same time: deletions are applied between batches on the graph's stream) and
// w is cleared afterwards.
#include <vector>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

__global__ void k_row_reset(int32_t* D, uint8_t* D8, int64_t* S, double* Dl, int64_t nv, int root, int32_t* order)
{
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nv; x += (int64_t)gridDim.x * blockDim.x) {
        const bool r = x == root;
        D[x] = r ? 0 : SBC_INF;
        D8[x] = r ? 0 : SBC_D8_INF;
        S[x] = r ? 1 : 0;
        Dl[x] = 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) order[0] = root;
}

__global__ void k_wide_forward(DevGraph G, int32_t* D, uint8_t* D8, int64_t* S, const int32_t* __restrict__ in, int nin,
                               int32_t* order, int* count, int L, unsigned long long* counters)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); i < nin; i += nwarps) {
        const int x = in[i];
        const int64_t rx = G.row[x];
        const int dx = G.deg[x];
        const int64_t sx = S[x];
        for (int s = lane; s < dx; s += 32) {
            const int k = G.col[rx + s];
            const int old = atomicCAS(&D[k], SBC_INF, L + 1);
            if (old == SBC_INF) {
                D8[k] = enc_d8(L + 1);
                order[atomicAdd(count, 1)] = k;
            }
            if (old == SBC_INF || old == L + 1) atomic_add_i64(&S[k], sx);
        }
        if (lane == 0) {
            atomicAdd(&counters[0], 1ull);
            atomicAdd(&counters[1], (unsigned long long)dx);
        }
    }
}

__global__ void k_wide_backward(DevGraph G, const int32_t* __restrict__ D, const int64_t* __restrict__ S, double* Dl,
                                double* w, const int32_t* __restrict__ lvl, int n, int L, unsigned long long* counters)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    for (int i = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5); i < n; i += nwarps) {
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
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        }
        if (lane == 0) {
            const double sx = (double)S[x];
            const double d = sx * sum;
            Dl[x] = d;
            w[x] = (d + 1.0) / sx;
            atomicAdd(&counters[0], 1ull);
            atomicAdd(&counters[1], (unsigned long long)dx);
        }
    }
}

__global__ void k_clear_w(double* w, const int32_t* __restrict__ order, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w[order[i]] = 0.0;
}

// Recomputes root row r of forest f; synchronous (one device-to-host read of
// the frontier size per level).
cudaError_t recompute_root_wide(sbc_forest* f, int r)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    const int64_t nv = f->nv;
    int32_t* D = f->d_dist + (size_t)r * nv;
    uint8_t* D8 = f->d_dist8 + (size_t)r * nv;
    int64_t* S = f->d_sigma + (size_t)r * nv;
    double* Dl = f->d_delta + (size_t)r * nv;
    int32_t* order = f->ws.qd;  // worker 0's slice
    double* w = f->ws.acc;
    int* count = f->d_nmov + 1;
    const int root = (int)f->h_roots[r];
    const DevGraph G = g->dev();
    const int grid = f->sm_count * 8;
    cudaError_t e;
    k_row_reset<<<grid, 256, 0, s>>>(D, D8, S, Dl, nv, root, order);
    static const int kOne = 1;
    if ((e = cudaMemcpyAsync(count, &kOne, sizeof(int), cudaMemcpyHostToDevice, s))) return e;
    std::vector<int> off = {0, 1};
    for (int L = 0;; ++L) {
        const int nin = off[L + 1] - off[L];
        if (nin == 0) break;
        k_wide_forward<<<grid, 256, 0, s>>>(G, D, D8, S, order + off[L], nin, order, count, L, f->d_counters);
        int c = 0;
        if ((e = cudaMemcpyAsync(&c, count, sizeof(int), cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
            return e;
        off.push_back(c);
    }
    // levels 0 .. off.size()-3 are non-empty; deepest first
    for (int L = (int)off.size() - 3; L >= 0; --L)
        k_wide_backward<<<grid, 256, 0, s>>>(G, D, S, Dl, w, order + off[L], off[L + 1] - off[L], L, f->d_counters);
    k_clear_w<<<grid, 256, 0, s>>>(w, order, off.back());
    return cudaGetLastError();
}

}  // namespace sbc
