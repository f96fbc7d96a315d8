// Static Brandes initialisation over K roots.
//
// Replaces BrandesApproxCaseParallel / BrandesSingleTree
// (src/streamingbc_init.c:60-84, :87-183).  One persistent CTA per worker slot
// takes roots from an atomic counter.  Per root:
//   forward   level-synchronous BFS; a frontier vertex pushes its sigma into
//             every neighbour on the next level (int64 atomics, so the sum is
//             exact and order-independent); the first visitor of a vertex
//             claims it with a CAS on dist and appends it to the next frontier.
//   backward  levels from deepest to 0, pull form: a vertex x sums
//             w[c] = (delta[c]+1)/sigma[c] over its children c (dist[c] =
//             dist[x]+1) and sets delta[x] = sigma[x] * sum; no global atomics.
// BC is then a column sum of delta over roots excluding each root itself
// (init.c:175-177), computed by k_bc_colsum in root order.
#include <climits>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

struct StaticArgs {
    DevGraph G;
    int64_t nv;
    int nk;
    const int64_t* roots;
    int32_t* dist;
    uint8_t* dist8;
    int64_t* sigma;
    double* delta;
    ScratchBase scr;
    int* work_counter;
    unsigned long long* counters;  // [0] vertices, [1] edges
};

template <int NT>
__global__ void __launch_bounds__(NT) k_static(StaticArgs A)
{
    __shared__ LbSmem<NT> sm;
    __shared__ int s_item, s_tail;
    __shared__ int64_t s_sig[NT];
    __shared__ double s_acc[NT];
    const int64_t nv = A.nv;
    Scratch W = A.scr.of(blockIdx.x, nv);
    if (threadIdx.x == 0) sm.walked_v = sm.walked_e = sm.scanned_e = 0;

    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int r = s_item;
        __syncthreads();
        if (r >= A.nk) break;
        int32_t* D = A.dist + (size_t)r * nv;
        uint8_t* D8 = A.dist8 + (size_t)r * nv;
        int64_t* Sg = A.sigma + (size_t)r * nv;
        double* Dl = A.delta + (size_t)r * nv;
        const int root = (int)A.roots[r];

        for (int64_t x = threadIdx.x; x < nv; x += NT) {
            D[x] = SBC_INF;
            D8[x] = SBC_D8_INF;
            Sg[x] = 0;
            Dl[x] = 0.0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            D[root] = 0;
            D8[root] = 0;
            Sg[root] = 1;
            W.qd[0] = root;
            W.lvl[0] = 0;
            W.lvl[1] = 1;
            s_tail = 1;
        }
        __syncthreads();

        // Forward: levels 0, 1, ...
        int L = 0, lo = 0, hi = 1;
        while (lo < hi) {
            lb_walk<NT>(
                A.G, INT_MAX, D, D8, W.qd + lo, hi - lo, nullptr, 0, sm,
                [&](int j, int x, int d) { s_sig[j] = Sg[x]; },
                [&](int j, int x, int k, int dk) {
                    if (dk == SBC_INF) {
                        int old = atomicCAS(&D[k], SBC_INF, L + 1);
                        if (old == SBC_INF) {
                            D8[k] = enc_d8(L + 1);
                            int p = atomicAdd(&s_tail, 1);
                            W.qd[p] = k;
                            dk = L + 1;
                        } else {
                            dk = old;
                        }
                    }
                    if (dk == L + 1) atomic_add_i64(&Sg[k], s_sig[j]);
                },
                NoPost());
            lo = hi;
            hi = s_tail;
            ++L;
            if (threadIdx.x == 0) W.lvl[L + 1] = hi;
        }
        __syncthreads();
        const int nlev = L;  // levels 0 .. nlev-1 are non-empty

        // Backward: deepest level first; w[x] lives in the worker's acc array.
        for (int l = nlev - 1; l >= 0; --l) {
            const int b0 = W.lvl[l], b1 = W.lvl[l + 1];
            lb_walk<NT>(
                A.G, INT_MAX, D, D8, W.qd + b0, b1 - b0, nullptr, 0, sm,
                [&](int j, int x, int d) { s_acc[j] = 0.0; },
                [&](int j, int x, int k, int dk) {
                    if (dk == l + 1) atomicAdd(&s_acc[j], W.acc[k]);
                },
                [&](int j, int x) {
                    double sx = (double)Sg[x];
                    double nd = sx * s_acc[j];
                    Dl[x] = nd;
                    W.acc[x] = (nd + 1.0) / sx;
                });
        }
        const int reached = W.lvl[nlev];
        for (int i = threadIdx.x; i < reached; i += NT) W.acc[W.qd[i]] = 0.0;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(&A.counters[0], sm.walked_v);
        atomicAdd(&A.counters[1], sm.walked_e);
        atomicAdd(&A.counters[4], sm.scanned_e);
    }
}

// bc[v] = sum over roots r (in root order) of delta[r][v], skipping v == root.
__global__ void k_bc_colsum(const double* __restrict__ delta, const int64_t* __restrict__ roots,
                            int nk, int64_t nv, double* __restrict__ bc)
{
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
         v += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int r = 0; r < nk; ++r) {
            double d = delta[(size_t)r * nv + v];
            if (roots[r] != v) s += d;
        }
        bc[v] = s;
    }
}

int static_workers_per_sm()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_static<256>, 256, 0);
    return n;
}

cudaError_t launch_static(sbc_forest* f)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(f->d_counter, 0, sizeof(int), s))) return e;
    StaticArgs A;
    A.G = g->dev();
    A.nv = f->nv;
    A.nk = (int)f->nk;
    A.roots = f->d_roots;
    A.dist = f->d_dist;
    A.dist8 = f->d_dist8;
    A.sigma = f->d_sigma;
    A.delta = f->d_delta;
    A.scr = f->scratch();
    A.work_counter = f->d_counter;
    A.counters = f->d_counters;
    // One worker slot per CTA: with few workers per SM, wider CTAs keep the SMs full.
    const int grid = (int)std::min<int64_t>(f->workers, f->nk);
    const int64_t per_sm = (f->workers + f->sm_count - 1) / f->sm_count;
    f->prof_begin(PROF_STATIC);
    if (per_sm <= 1) k_static<1024><<<grid, 1024, 0, s>>>(A);
    else if (per_sm <= 2) k_static<512><<<grid, 512, 0, s>>>(A);
    else k_static<256><<<grid, 256, 0, s>>>(A);
    f->prof_end(PROF_STATIC);
    if ((e = cudaGetLastError())) return e;
    int bgrid = (int)std::min<int64_t>((f->nv + 255) / 256, (int64_t)f->sm_count * 8);
    if (bgrid < 1) bgrid = 1;
    k_bc_colsum<<<bgrid, 256, 0, s>>>(f->d_delta, f->d_roots, (int)f->nk, f->nv, f->d_bc);
    return cudaGetLastError();
}

}  // namespace sbc
