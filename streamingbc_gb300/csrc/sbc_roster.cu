// Rosters: per root, the members of each small level of its tree.
//
// In the reference a vertex finds its parents by scanning its whole adjacency
// for neighbours one level up (src/streamingbc_internal.c:138-211, :427-545).
// For a root far from the graph's hubs (a degree-1 vertex of an R-MAT graph,
// say), the hubs sit at level 3 of its tree under a level 2 of a few dozen
// vertices, and every insertion that reaches them scans hub adjacencies of
// 10^4-10^5 slots to find those few parents.  A roster lists the members of a
// level with at most kRosterCap vertices; the update kernel then finds the
// parents of such a vertex by binary search for each roster member in its
// sorted adjacency (same parents, same results).
//
// Levels only shrink under insertions, and a vertex only moves to a shallower
// level (in a re-levelling descent), which appends it to its new level's
// roster; its old entry is left in place and marked stale.  Rosters are
// therefore supersets of their levels, readers check distances, and
// k_roster_compact drops stale entries after each batch.
//   k_roster_build    CTA per root: members of levels 2..kRosterLevels-1 whose
//                     level histogram count fits a roster (after static init)
//   k_roster_compact  warp per (root, level) roster marked stale (the _group
//                     form: for several forests in one launch)
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

__global__ void __launch_bounds__(256) k_roster_build(const uint8_t* __restrict__ dist8, int64_t nv,
                                                      const int32_t* __restrict__ hist, int32_t* __restrict__ roster,
                                                      int32_t* __restrict__ roster_n, int32_t* __restrict__ dirty,
                                                      const int* __restrict__ list, const int* __restrict__ nlist)
{
    __shared__ int cnt[kRosterLevels];
    __shared__ int ok[kRosterLevels];
    if (list && (int)blockIdx.x >= *nlist) return;
    const size_t r = list ? (size_t)list[blockIdx.x] : blockIdx.x;
    const int32_t* H = hist + r * kHistLevels;
    if (threadIdx.x < kRosterLevels) {
        cnt[threadIdx.x] = 0;
        ok[threadIdx.x] = threadIdx.x >= 2 && H[threadIdx.x] <= kRosterCap;
    }
    __syncthreads();
    const uint8_t* D8 = dist8 + r * nv;
    int32_t* R = roster + r * kRosterLevels * kRosterCap;
    for (int64_t v = threadIdx.x; v < nv; v += blockDim.x) {
        const int d = D8[v];
        if (d < kRosterLevels && ok[d]) {
            const int p = atomicAdd(&cnt[d], 1);
            if (p < kRosterCap) R[d * kRosterCap + p] = (int32_t)v;
        }
    }
    __syncthreads();
    if (threadIdx.x < kRosterLevels) {
        roster_n[r * kRosterLevels + threadIdx.x] = ok[threadIdx.x] ? min(cnt[threadIdx.x], kRosterCap + 1)
                                                                    : kRosterCap + 1;
        dirty[r * kRosterLevels + threadIdx.x] = 0;
    }
}

// Warp w = root * kRosterLevels + level drops the stale entries of its roster.
__device__ __forceinline__ void compact_one(const uint8_t* __restrict__ dist8, int64_t nv,
                                            int32_t* __restrict__ roster, int32_t* __restrict__ roster_n,
                                            int32_t* __restrict__ dirty, int w, int lane)
{
    if (!dirty[w]) return;  // warp-uniform
    const int n = roster_n[w];
    if (n > kRosterCap) return;
    const int level = w % kRosterLevels;
    const uint8_t* D8 = dist8 + (size_t)(w / kRosterLevels) * nv;
    int32_t* R = roster + (size_t)w * kRosterCap;
    int kept = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const int v = i < n ? R[i] : -1;
        const bool keep = v >= 0 && D8[v] == level;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        __syncwarp();  // every lane has read its entry before any is overwritten
        if (keep) R[kept + __popc(m & ((1u << lane) - 1u))] = v;
        kept += __popc(m);
        __syncwarp();
    }
    if (lane == 0) {
        roster_n[w] = kept;
        dirty[w] = 0;
    }
}

__global__ void __launch_bounds__(256) k_roster_compact(const uint8_t* __restrict__ dist8, int64_t nv, int nk,
                                                        int32_t* __restrict__ roster, int32_t* __restrict__ roster_n,
                                                        int32_t* __restrict__ dirty)
{
    const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    if (w >= nk * kRosterLevels) return;
    compact_one(dist8, nv, roster, roster_n, dirty, w, threadIdx.x & 31);
}

// Several forests in one launch (the members of a group batch).
struct RosterForest {
    const uint8_t* dist8;
    int64_t nv;
    int32_t* roster;
    int32_t* roster_n;
    int32_t* dirty;
};

struct RosterGroupArgs {
    RosterForest f[kMaxGroup];
    int64_t wbase[kMaxGroup + 1];  // prefix sums of nk * kRosterLevels
    int nf;
};

__global__ void __launch_bounds__(256) k_roster_compact_group(const __grid_constant__ RosterGroupArgs A)
{
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (w >= A.wbase[A.nf]) return;
    int lo = 0, hi = A.nf - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.wbase[mid] <= w) lo = mid;
        else hi = mid - 1;
    }
    const RosterForest& F = A.f[lo];
    compact_one(F.dist8, F.nv, F.roster, F.roster_n, F.dirty, (int)(w - A.wbase[lo]), threadIdx.x & 31);
}

cudaError_t launch_roster_compact_forests(sbc_forest* const* fs, int nf, cudaStream_t s)
{
    for (int at = 0; at < nf; at += kMaxGroup) {
        RosterGroupArgs A;
        A.nf = 0;
        A.wbase[0] = 0;
        for (int j = at; j < nf && j < at + kMaxGroup; ++j) {
            sbc_forest* f = fs[j];
            if (!f->d_roster) continue;
            RosterForest& F = A.f[A.nf];
            F.dist8 = f->d_dist8;
            F.nv = f->nv;
            F.roster = f->d_roster;
            F.roster_n = f->d_roster_n;
            F.dirty = f->d_roster_dirty;
            A.wbase[A.nf + 1] = A.wbase[A.nf] + f->nk * kRosterLevels;
            ++A.nf;
        }
        if (A.nf == 0) continue;
        k_roster_compact_group<<<(int)((A.wbase[A.nf] * 32 + 255) / 256), 256, 0, s>>>(A);
        cudaError_t e = cudaGetLastError();
        if (e) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_roster_build(sbc_forest* f) { return launch_roster_build_list(f, nullptr, nullptr); }

cudaError_t launch_roster_build_list(sbc_forest* f, const int* d_list, const int* d_nlist)
{
    if (!f->d_roster) return cudaSuccess;
    k_roster_build<<<(int)f->nk, 256, 0, f->g->stream>>>(f->d_dist8, f->nv, f->d_lvlhist, f->d_roster,
                                                          f->d_roster_n, f->d_roster_dirty, d_list, d_nlist);
    return cudaGetLastError();
}

cudaError_t launch_roster_compact(sbc_forest* f, cudaStream_t s)
{
    if (!f->d_roster) return cudaSuccess;
    const int64_t warps = f->nk * kRosterLevels;
    k_roster_compact<<<(int)((warps * 32 + 255) / 256), 256, 0, s>>>(
        f->d_dist8, f->nv, (int)f->nk, f->d_roster, f->d_roster_n, f->d_roster_dirty);
    return cudaGetLastError();
}

}  // namespace sbc
