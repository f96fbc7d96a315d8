// Level-2 parent masks (see kL1Max in sbc_internal.cuh).
//
// A level-2 vertex's parents are its neighbours among the root's neighbours.
// The insertion ascent (src/streamingbc_internal.c:138-211, :427-545) finds a
// vertex's parents by testing neighbour levels; at level 2 of a root with few
// neighbours that test costs a scan of hub adjacencies on every job, though
// the answer depends on the graph alone.  Here, for every root with at most
// kL1Max neighbours, mask[r][x] keeps the answer as a bit set over the root's
// neighbour list:
//   k_l2mask_build   per root (CTA): the neighbour list, the row cleared, then
//                    every neighbour i ORs bit i into the masks of its own
//                    neighbours.  After static init for all roots; later for
//                    the roots flagged by a change of the root's own edges.
//   k_l2mask_insert  after a batch's appends (thread per root x insertion):
//                    slot x -> z with z the root's neighbour i sets bit i of
//                    mask[r][x]; an edge at the root flags the root.
//   k_l2mask_remove  after an edge removal (thread per root): clears the bits
//                    of the removed slots; an edge at the root flags it
//                    (the _batch form: thread per (root, removal)).
//   *_group          the same for several forests in one launch per step.
// Masks describe the edges that existed when a batch began; the update adds
// the edges its batch appended before the job (visible by seq) itself.
#include <algorithm>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

__device__ __forceinline__ int l1_index(const int32_t* C, int n, int z)
{
    for (int i = 0; i < n; ++i)
        if (C[i] == z) return i;
    return -1;
}

__device__ __forceinline__ void flag_rebuild(int32_t* flag, int32_t* list, int32_t* cnt, int r)
{
    if (atomicExch(&flag[r], 1) == 0) list[atomicAdd(cnt, 1)] = r;
}

// Builds the masks of root r (one CTA).  Every slot of the root and of its
// neighbours is an edge (called between batches: deg0 == deg).
__device__ __forceinline__ void build_root(DevGraph G, const int64_t* roots, uint32_t* mask, int32_t* cand,
                                           int32_t* l1n, int r)
{
    const int64_t nv = G.nv;
    const int root = (int)roots[r];
    const int rdeg = G.deg[root];
    uint32_t* M = mask + (size_t)r * nv;
    int32_t* C = cand + (size_t)r * kL1Max;
    if (rdeg > kL1Max) {
        if (threadIdx.x == 0) l1n[r] = -1;
        return;
    }
    for (int64_t x = threadIdx.x; x < nv; x += blockDim.x) M[x] = 0u;
    const int64_t rr = G.row[root];
    for (int i = threadIdx.x; i < rdeg; i += blockDim.x) C[i] = G.col[rr + i];
    __syncthreads();
    for (int i = 0; i < rdeg; ++i) {
        const int y = C[i];
        const int64_t ry = G.row[y];
        const int dy = G.deg[y];
        for (int s = threadIdx.x; s < dy; s += blockDim.x) atomicOr(&M[G.col[ry + s]], 1u << i);
    }
    if (threadIdx.x == 0) l1n[r] = rdeg;
}

__global__ void __launch_bounds__(512) k_l2mask_build(DevGraph G, const int64_t* roots, int nk, uint32_t* mask,
                                                     int32_t* cand, int32_t* l1n, int32_t* flag,
                                                     const int32_t* list, const int32_t* cnt)
{
    const int n = list ? *cnt : nk;
    for (int item = blockIdx.x; item < n; item += gridDim.x) {
        const int r = list ? list[item] : item;
        build_root(G, roots, mask, cand, l1n, r);
        if (threadIdx.x == 0 && flag) flag[r] = 0;
        __syncthreads();
    }
}

// The masks of root r after the append of insertion (u, v).
__device__ __forceinline__ void insert_one(const int64_t* roots, int r, int u, int v, int directed, int64_t nv,
                                           uint32_t* mask, const int32_t* cand, const int32_t* l1n, int32_t* flag,
                                           int32_t* list, int32_t* cnt)
{
    const int root = (int)roots[r];
    if (u == root || v == root) {
        flag_rebuild(flag, list, cnt, r);
        return;
    }
    const int c = l1n[r];
    if (c < 0) return;
    const int32_t* C = cand + (size_t)r * kL1Max;
    uint32_t* M = mask + (size_t)r * nv;
    const int bv = l1_index(C, c, v);  // slot u -> v
    if (bv >= 0) atomicOr(&M[u], 1u << bv);
    if (!directed) {
        const int bu = l1_index(C, c, u);  // slot v -> u
        if (bu >= 0) atomicOr(&M[v], 1u << bu);
    }
}

__global__ void k_l2mask_insert(const int64_t* __restrict__ roots, int nk, int n, const int32_t* __restrict__ iu,
                                const int32_t* __restrict__ iv, const int32_t* __restrict__ ok, int directed,
                                int64_t nv, uint32_t* mask, const int32_t* __restrict__ cand,
                                const int32_t* __restrict__ l1n, int32_t* flag, int32_t* list, int32_t* cnt)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nk * n) return;
    const int r = (int)(t / n), i = (int)(t % n);
    if (ok[i] <= 0) return;
    insert_one(roots, r, iu[i], iv[i], directed, nv, mask, cand, l1n, flag, list, cnt);
}

// Several forests in one launch per step (the forests on the graphs of a
// group batch): one entry per forest with its staged insertions.
struct MaskForest {
    DevGraph G;
    const int64_t* roots;
    uint32_t* mask;
    int32_t* cand;
    int32_t* l1n;
    int32_t* flag;
    int32_t* list;
    int32_t* cnt;
    const int32_t* iu;
    const int32_t* iv;
    const int32_t* ok;
    int nk;
    int n;
};

struct MaskGroupArgs {
    MaskForest f[kMaxGroup];
    int64_t base[kMaxGroup + 1];  // prefix sums of nk * n
    int nf;
    int directed;
};

// One thread per (forest, root, insertion).
__global__ void k_l2mask_insert_group(const __grid_constant__ MaskGroupArgs A)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= A.base[A.nf]) return;
    int lo = 0, hi = A.nf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.base[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const MaskForest& F = A.f[lo];
    const int64_t local = t - A.base[lo];
    const int r = (int)(local / F.n), i = (int)(local % F.n);
    if (F.ok[i] <= 0) return;
    insert_one(F.roots, r, F.iu[i], F.iv[i], A.directed, F.G.nv, F.mask, F.cand, F.l1n, F.flag, F.list, F.cnt);
}

// The flagged roots of every forest, CTA per root.
__global__ void __launch_bounds__(512) k_l2mask_build_group(const __grid_constant__ MaskGroupArgs A)
{
    for (int j = 0; j < A.nf; ++j) {
        const MaskForest& F = A.f[j];
        const int n = *F.cnt;
        for (int item = blockIdx.x; item < n; item += gridDim.x) {
            const int r = F.list[item];
            build_root(F.G, F.roots, F.mask, F.cand, F.l1n, r);
            if (threadIdx.x == 0) F.flag[r] = 0;
            __syncthreads();
        }
    }
}

__global__ void k_l2mask_reset_group(const __grid_constant__ MaskGroupArgs A)
{
    if ((int)threadIdx.x < A.nf) *A.f[threadIdx.x].cnt = 0;
}

__global__ void k_l2mask_remove(const int64_t* __restrict__ roots, int nk, int u, int v, int directed,
                                const int* __restrict__ removed, int64_t nv, uint32_t* mask,
                                const int32_t* __restrict__ cand, const int32_t* __restrict__ l1n, int32_t* flag,
                                int32_t* list, int32_t* cnt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nk || *removed != 1) return;
    const int root = (int)roots[r];
    if (u == root || v == root) {
        flag_rebuild(flag, list, cnt, r);
        return;
    }
    const int c = l1n[r];
    if (c < 0) return;
    const int32_t* C = cand + (size_t)r * kL1Max;
    uint32_t* M = mask + (size_t)r * nv;
    const int bv = l1_index(C, c, v);
    if (bv >= 0) atomicAnd(&M[u], ~(1u << bv));
    if (!directed) {
        const int bu = l1_index(C, c, u);
        if (bu >= 0) atomicAnd(&M[v], ~(1u << bu));
    }
}

// After a batch of removals (undirected; code[i] == 1: removed): thread per
// (root, deletion), as k_l2mask_remove does for one.
__global__ void k_l2mask_remove_batch(const int64_t* __restrict__ roots, int nk, int n, const int32_t* __restrict__ iu,
                                      const int32_t* __restrict__ iv, const int32_t* __restrict__ code, int64_t nv,
                                      uint32_t* mask, const int32_t* __restrict__ cand,
                                      const int32_t* __restrict__ l1n, int32_t* flag, int32_t* list, int32_t* cnt)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)nk * n) return;
    const int r = (int)(t / n), i = (int)(t % n);
    if (code[i] != 1) return;
    const int u = iu[i], v = iv[i];
    const int root = (int)roots[r];
    if (u == root || v == root) {
        flag_rebuild(flag, list, cnt, r);
        return;
    }
    const int c = l1n[r];
    if (c < 0) return;
    const int32_t* C = cand + (size_t)r * kL1Max;
    uint32_t* M = mask + (size_t)r * nv;
    const int bv = l1_index(C, c, v);
    if (bv >= 0) atomicAnd(&M[u], ~(1u << bv));
    const int bu = l1_index(C, c, u);
    if (bu >= 0) atomicAnd(&M[v], ~(1u << bu));
}

namespace {

// Rebuilds the flagged roots, then empties the list.
cudaError_t rebuild_flagged(sbc_forest* f, cudaStream_t s)
{
    k_l2mask_build<<<64, 512, 0, s>>>(f->g->dev(), f->d_roots, (int)f->nk, f->d_l2mask, f->d_l1cand, f->d_l1n,
                                      f->d_l2flag, f->d_l2list, f->d_l2cnt);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    return cudaMemsetAsync(f->d_l2cnt, 0, sizeof(int32_t), s);
}

}  // namespace

cudaError_t launch_l2mask_build_all(sbc_forest* f)
{
    if (!f->d_l2mask) return cudaSuccess;
    const int grid = (int)std::min<int64_t>(f->nk, (int64_t)f->sm_count * 4);
    k_l2mask_build<<<grid, 512, 0, f->g->stream>>>(f->g->dev(), f->d_roots, (int)f->nk, f->d_l2mask, f->d_l1cand,
                                                   f->d_l1n, nullptr, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_l2mask_insert_forest(sbc_forest* f, int n, bool directed, cudaStream_t s)
{
    if (!f->d_l2mask || n <= 0) return cudaSuccess;
    sbc_graph* g = f->g;
    const int64_t threads = f->nk * (int64_t)n;
    k_l2mask_insert<<<(int)((threads + 255) / 256), 256, 0, s>>>(
        f->d_roots, (int)f->nk, n, g->d_ins, g->d_ins + g->ins_capacity, g->d_ins + 2 * g->ins_capacity,
        directed ? 1 : 0, f->nv, f->d_l2mask, f->d_l1cand, f->d_l1n, f->d_l2flag, f->d_l2list, f->d_l2cnt);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    return rebuild_flagged(f, s);
}

cudaError_t launch_l2mask_insert_forests(sbc_forest* const* fs, const int* counts, int nf, bool directed,
                                        cudaStream_t s)
{
    for (int at = 0; at < nf; at += kMaxGroup) {
        MaskGroupArgs A;
        A.nf = 0;
        A.directed = directed ? 1 : 0;
        A.base[0] = 0;
        for (int j = at; j < std::min(nf, at + kMaxGroup); ++j) {
            sbc_forest* f = fs[j];
            if (!f->d_l2mask || counts[j] <= 0) continue;
            sbc_graph* g = f->g;
            MaskForest& F = A.f[A.nf];
            F.G = g->dev();
            F.roots = f->d_roots;
            F.mask = f->d_l2mask;
            F.cand = f->d_l1cand;
            F.l1n = f->d_l1n;
            F.flag = f->d_l2flag;
            F.list = f->d_l2list;
            F.cnt = f->d_l2cnt;
            F.iu = g->d_ins;
            F.iv = g->d_ins + g->ins_capacity;
            F.ok = g->d_ins + 2 * g->ins_capacity;
            F.nk = (int)f->nk;
            F.n = counts[j];
            A.base[A.nf + 1] = A.base[A.nf] + f->nk * (int64_t)counts[j];
            ++A.nf;
        }
        if (A.nf == 0) continue;
        const int64_t threads = A.base[A.nf];
        k_l2mask_insert_group<<<(int)((threads + 255) / 256), 256, 0, s>>>(A);
        cudaError_t e = cudaGetLastError();
        if (e) return e;
        k_l2mask_build_group<<<64, 512, 0, s>>>(A);
        if ((e = cudaGetLastError())) return e;
        k_l2mask_reset_group<<<1, kMaxGroup, 0, s>>>(A);
        if ((e = cudaGetLastError())) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_l2mask_insert(sbc_graph* g, int n, bool directed)
{
    for (sbc_forest* f : g->forests) {
        cudaError_t e = launch_l2mask_insert_forest(f, n, directed, g->stream);
        if (e) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_l2mask_remove_batch(sbc_graph* g, int n)
{
    for (sbc_forest* f : g->forests) {
        if (!f->d_l2mask || n <= 0) continue;
        const int64_t threads = f->nk * (int64_t)n;
        k_l2mask_remove_batch<<<(int)((threads + 255) / 256), 256, 0, g->stream>>>(
            f->d_roots, (int)f->nk, n, g->d_ins, g->d_ins + g->ins_capacity, g->d_ins + 2 * g->ins_capacity, f->nv,
            f->d_l2mask, f->d_l1cand, f->d_l1n, f->d_l2flag, f->d_l2list, f->d_l2cnt);
        cudaError_t e = cudaGetLastError();
        if (e) return e;
        if ((e = rebuild_flagged(f, g->stream))) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_l2mask_remove(sbc_graph* g, int u, int v, bool directed, const int* d_removed)
{
    for (sbc_forest* f : g->forests) {
        if (!f->d_l2mask) continue;
        k_l2mask_remove<<<(int)((f->nk + 255) / 256), 256, 0, g->stream>>>(
            f->d_roots, (int)f->nk, u, v, directed ? 1 : 0, d_removed, f->nv, f->d_l2mask, f->d_l1cand, f->d_l1n,
            f->d_l2flag, f->d_l2list, f->d_l2cnt);
        cudaError_t e = cudaGetLastError();
        if (e) return e;
        if ((e = rebuild_flagged(f, g->stream))) return e;
    }
    return cudaSuccess;
}

}  // namespace sbc
