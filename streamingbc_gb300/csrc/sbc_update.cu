// Incremental BC update for edge insertions over K roots.
//
// Replaces insertEdgeStreamingBC's COARSE loop (src/streamingbc.c:88-226) and
// the two insertion cases it dispatches to:
//   |d| == 1  addEdgeWithoutMovementBrandes  (src/streamingbc_internal.c:11-248)
//   |d|  > 1  moveUpTreeBrandes              (src/streamingbc_internal.c:251-603)
// with the same parent-free method: parents/children are found by comparing
// neighbour distances, and the case is picked by d(r,u) - d(r,v).
//
// Kernels:
//   k_classify  one thread per root: a root stays in the batch's worklist iff
//               some insertion of the batch joins two different levels at the
//               batch start (otherwise no insertion of the batch can change
//               the root's state, so it is culled for the whole batch).
//   k_update    persistent CTAs; each takes a root from the worklist and applies
//               every insertion of the batch to it in order.  One insertion on
//               one root is a "job":
//     descent  level-synchronous BFS from the deeper endpoint b.  |d|==1:
//              children (dist = level+1) gain diffPath; |d|>1: neighbours with
//              old dist >= new level+1 join the next level (moved if strictly
//              deeper before) and gain diffPath.  A vertex is claimed for a
//              level with a CAS on its step tag; diffPath sums are int64 atomics.
//     re-level (|d|>1) every descent vertex gets new dist = new level of its step.
//     ascent   new levels from deepest to 0.  Per level: phase A walks the
//              descent vertices, phase B the ascent-only vertices claimed for
//              this level (parents found at level+1, and, for |d|>1, same-level
//              ex-parents of moved vertices found in phase A).  Each vertex's
//              new delta is final when its level starts; it pushes
//              newsigma[k]*(newdelta[x]+1)/newsigma[x] into each parent k, minus
//              its old contribution when k is ascent-only (except the new edge),
//              adds newdelta-olddelta to BC, and commits sigma/delta in place.
//     reset    scratch of every touched vertex is cleared (O(touched)).
// Results are exact for dist/sigma (integer atomics); BC/delta differ from the
// reference only by floating-point summation order.
#include <climits>
#include <vector>
#include "sbc_gb300.h"
#include "sbc_host.h"
#include "sbc_internal.cuh"
#include "sbc_update_job.cuh"

namespace sbc {

struct UpdateArgs {
    ForestSlot f;
    ScratchBase scr;
    int all_visible;
    int del_u, del_v;  // k_delete: the deleted edge
    int* mov;          // k_delete: roots left to a recompute
    int* nmov;
    int move_down;     // k_delete_batch: lost-parent roots move down (else recompute)
    int* dirty;        // k_delete_batch: roots recomputed after the launch
    int* dlist;
    int* dcnt;
    const int* worklist;
    const int* nwork;
    int* work_counter;
    unsigned long long* counters;  // vertices, edges, case1, case2, scanned
};

template <int NT, int MINB, int ILP>
__global__ void __launch_bounds__(NT, MINB) k_update(const __grid_constant__ UpdateArgs A)
{
    __shared__ UpdSmem<NT> sm;
    const Scratch W = A.scr.of(blockIdx.x, A.f.G.nv);
    const int nwork = *A.nwork;
    reset_counters<NT>(sm);

    for (;;) {
        if (threadIdx.x == 0) sm.item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int item = sm.item;
        __syncthreads();
        if (item >= nwork) break;
        process_root<NT, ILP>(A.f, sm, W, A.worklist[item], A.all_visible != 0);
    }
    flush_counters<NT>(sm, A.counters);
}

// Deletions (one launch per deletion, after k_classify_delete): its own
// kernel, so the insertion kernel's code and registers are untouched; any
// launch shape fits the forest's worker scratch, since it only indexes worker
// slots below its grid.  Worklist entries carry kLostRoot for roots whose
// deeper endpoint lost its last parent.
template <int NT, int MINB, int ILP>
__global__ void __launch_bounds__(NT, MINB) k_delete(const __grid_constant__ UpdateArgs A)
{
    __shared__ UpdSmem<NT> sm;
    const Scratch W = A.scr.of(blockIdx.x, A.f.G.nv);
    const int nwork = *A.nwork;
    reset_counters<NT>(sm);
    for (;;) {
        if (threadIdx.x == 0) sm.item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int item = sm.item;
        __syncthreads();
        if (item >= nwork) break;
        const int w = A.worklist[item];
        process_deletion<NT, ILP>(A.f, sm, W, w & ~kLostRoot, A.del_u, A.del_v, (w & kLostRoot) != 0, A.mov,
                                  A.nmov);
    }
    flush_counters<NT>(sm, A.counters);
}

// A batch of deletions in one persistent launch: a CTA per active root runs
// the batch's deletions in order on it (process_root_deletions).
template <int NT, int MINB, int ILP>
__global__ void __launch_bounds__(NT, MINB) k_delete_batch(const __grid_constant__ UpdateArgs A)
{
    __shared__ UpdSmem<NT> sm;
    const Scratch W = A.scr.of(blockIdx.x, A.f.G.nv);
    const int nwork = *A.nwork;
    reset_counters<NT>(sm);
    for (;;) {
        if (threadIdx.x == 0) sm.item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int item = sm.item;
        __syncthreads();
        if (item >= nwork) break;
        process_root_deletions<NT, ILP>(A.f, sm, W, A.worklist[item], A.move_down != 0, A.dirty, A.dlist, A.dcnt);
    }
    flush_counters<NT>(sm, A.counters);
}

// Roots a batch of deletions can change: some removed edge joins two
// different levels of the root's tree as the batch begins (while every
// deletion so far was same-level the root is unchanged, so a root none of
// whose deletions is different-level stays unchanged).  Warp per root, lanes
// over the deletions.
__global__ void k_classify_delete_batch(const int32_t* __restrict__ dist, int64_t nv, int nk, int n,
                                        const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                                        const int32_t* __restrict__ code, int* __restrict__ worklist,
                                        int* __restrict__ nwork)
{
    const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= nk) return;
    const int32_t* D = dist + (size_t)r * nv;
    bool active = false;
    for (int base = 0; base < n && !active; base += 32) {
        const int i = base + lane;
        active = __any_sync(0xffffffffu, i < n && code[i] == 1 && D[iu[i]] != D[iv[i]]);
    }
    if (lane == 0 && active) worklist[atomicAdd(nwork, 1)] = r;
}

__global__ void k_classify(const int32_t* __restrict__ dist, int64_t nv, int nk, int nins,
                           const int32_t* __restrict__ iu, const int32_t* __restrict__ iv,
                           const int32_t* __restrict__ ok, int* __restrict__ worklist, int* __restrict__ nwork)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nk) return;
    const int32_t* D = dist + (size_t)r * nv;
    bool active = false;
    for (int i = 0; i < nins && !active; ++i)
        if (ok[i] > 0 && D[iu[i]] != D[iv[i]]) active = true;
    if (active) {
        int p = atomicAdd(nwork, 1);
        worklist[p] = r;
    }
}

// Launch shapes of k_update: threads per persistent CTA and the minimum number
// of resident CTAs per SM the compiler must fit (which caps registers).  More
// resident CTAs means more roots in flight and more outstanding gathers; more
// threads per CTA means faster walks over one root's frontiers.
template <int NT, int MINB, int ILP>
void launch_variant(const UpdateArgs& A, int grid, cudaStream_t s)
{
    k_update<NT, MINB, ILP><<<grid, NT, 0, s>>>(A);
}

template <int NT, int MINB, int ILP>
int occupancy_variant()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_update<NT, MINB, ILP>, NT, 0);
    return n;
}

struct UpdateVariant {
    int threads, min_blocks, ilp;
    void (*launch)(const UpdateArgs&, int, cudaStream_t);
    int (*occupancy)();
};

static const UpdateVariant kVariants[] = {
    {256, 4, 4, launch_variant<256, 4, 4>, occupancy_variant<256, 4, 4>},
    {256, 5, 4, launch_variant<256, 5, 4>, occupancy_variant<256, 5, 4>},
    {256, 6, 4, launch_variant<256, 6, 4>, occupancy_variant<256, 6, 4>},
    {128, 8, 4, launch_variant<128, 8, 4>, occupancy_variant<128, 8, 4>},
    {128, 10, 4, launch_variant<128, 10, 4>, occupancy_variant<128, 10, 4>},
    {512, 2, 4, launch_variant<512, 2, 4>, occupancy_variant<512, 2, 4>},
    {512, 1, 4, launch_variant<512, 1, 4>, occupancy_variant<512, 1, 4>},
    {1024, 1, 4, launch_variant<1024, 1, 4>, occupancy_variant<1024, 1, 4>},
    // one or two warps per root (coarse grain): many roots in flight, for
    // graphs whose per-root touched sets are a few hundred vertices
    {64, 16, 4, launch_variant<64, 16, 4>, occupancy_variant<64, 16, 4>},
    {32, 32, 4, launch_variant<32, 32, 4>, occupancy_variant<32, 32, 4>},
    // deeper (8) or shallower (2) gather pipelines per thread
    {1024, 1, 8, launch_variant<1024, 1, 8>, occupancy_variant<1024, 1, 8>},
    {512, 2, 8, launch_variant<512, 2, 8>, occupancy_variant<512, 2, 8>},
    {128, 8, 2, launch_variant<128, 8, 2>, occupancy_variant<128, 8, 2>},
    {256, 4, 2, launch_variant<256, 4, 2>, occupancy_variant<256, 4, 2>},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);
// 1024 threads x 1 CTA per SM measured fastest on R-MAT scale 20, K = 1024
// (531 insertions/s against 413 for 512x2 and 281 for 256x4): with one root in
// flight per SM, the in-flight one-byte distance rows (152 x 1 MB) about fit
// the 129 MB L2, so repeated scans of the same hub ancestors within a root's
// batch hit L2 instead of HBM.
constexpr int kDefaultVariant = 7;

// Deletion of (u, v), already removed from the adjacency: warp per root.  A
// root whose endpoints sit on the same level (or are both unreachable) is
// unaffected; otherwise the deeper endpoint b either keeps a parent (a
// neighbour one level up) -- sigma-only update -- or has none and its subtree
// moves down (the reference's split, src/streamingbc.c:300-345); the second
// kind joins the work list flagged with kLostRoot (move_down) or the
// recompute list mov.
__global__ void k_classify_delete(const int32_t* __restrict__ dist, int64_t nv, int nk, DevGraph G, int u, int v,
                                  const int* __restrict__ removed, const int* __restrict__ dirty,
                                  int* __restrict__ adj, int* __restrict__ nadj, int* __restrict__ mov,
                                  int* __restrict__ nmov, int move_down, unsigned long long* counters)
{
    const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    // a root left for the batch's final recompute is no longer followed
    if (r >= nk || *removed != 1 || dirty[r]) return;
    const int32_t* D = dist + (size_t)r * nv;
    const int du = D[u], dv = D[v];
    if (du == dv) return;
    const int b = du > dv ? u : v;
    const int lb = du > dv ? du : dv;
    const int64_t rb = G.row[b];
    const int db = G.deg[b];
    bool parent = false;
    for (int base = 0; base < db && !parent; base += 32) {
        const int s = base + lane;
        parent = __any_sync(0xffffffffu, s < db && D[G.col[rb + s]] == lb - 1);
    }
    if (lane == 0) {
        if (parent || move_down) adj[atomicAdd(nadj, 1)] = parent ? r : (r | kLostRoot);
        else mov[atomicAdd(nmov, 1)] = r;
        if (!parent) atomicAdd(&counters[3], 1ull);
    }
}

// bc[v] += sign * delta[r][v] (v != root) for every root r of the list.
__global__ void k_bc_rows(const double* __restrict__ delta, const int64_t* __restrict__ roots,
                          const int* __restrict__ list, const int* __restrict__ nlist, int64_t nv, double* bc,
                          double sign)
{
    const int n = *nlist;
    for (int i = blockIdx.y; i < n; i += gridDim.y) {
        const int r = list[i];
        const int64_t root = roots[r];
        const double* Dl = delta + (size_t)r * nv;
        for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nv; x += (int64_t)gridDim.x * blockDim.x) {
            const double d = Dl[x];
            if (d != 0.0 && x != root) atomicAdd(&bc[x], sign * d);
        }
    }
}

int update_variant_count() { return kNumVariants; }
int update_default_variant() { return kDefaultVariant; }
int update_variant_threads(int v) { return kVariants[v].threads; }

int update_workers_per_sm(int v) { return kVariants[v].occupancy(); }

cudaError_t launch_update(sbc_forest* f, int n, bool all_visible)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    cudaError_t e;
    const int32_t* iu = g->d_ins;
    const int32_t* iv = g->d_ins + g->ins_capacity;
    const int32_t* ok = g->d_ins + 2 * g->ins_capacity;
    f->prof_begin(PROF_CLASSIFY);
    // cost-model features / ordered worklist (when the forest logs or is
    // scheduled by the model), else the static classify order
    bool ordered = false;
    if ((e = launch_schedule(f, n, &ordered))) return e;
    if (!ordered) {
        if ((e = cudaMemsetAsync(f->d_nwork, 0, 2 * sizeof(int), s))) return e;  // nwork, counter
        k_classify<<<(int)((f->nk + 255) / 256), 256, 0, s>>>(f->d_dist, f->nv, (int)f->nk, n, iu, iv, ok,
                                                              f->d_worklist, f->d_nwork);
    }
    f->prof_end(PROF_CLASSIFY);
    if ((e = cudaGetLastError())) return e;
    UpdateArgs A;
    A.f = forest_slot(f, n);
    if (f->model && f->model->logging) A.f.cost_log = f->model->d_cost_log;
    A.scr = f->scratch();
    A.all_visible = all_visible ? 1 : 0;
    A.del_u = A.del_v = 0;
    A.mov = A.nmov = nullptr;
    A.worklist = f->d_worklist;
    A.nwork = f->d_nwork;
    A.work_counter = f->d_counter;
    A.counters = f->d_counters;
    const int grid = (int)std::min<int64_t>(f->workers, f->nk);
    f->prof_begin(PROF_UPDATE);
    kVariants[f->variant].launch(A, grid, s);
    f->prof_end(PROF_UPDATE);
    if ((e = cudaGetLastError())) return e;
    if ((e = launch_log_append(f, n))) return e;
    return launch_roster_compact(f, s);
}

// The roots of the deletion's recompute list join the batch's dirty list.
__global__ void k_mark_dirty(const int* __restrict__ mov, const int* __restrict__ nmov, int* dirty, int* dlist,
                             int* dcnt)
{
    const int n = *nmov;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = mov[i];
        dirty[r] = 1;
        dlist[atomicAdd(dcnt, 1)] = r;
    }
}

__global__ void k_clear_dirty(const int* __restrict__ dlist, const int* __restrict__ dcnt, int* dirty)
{
    const int n = *dcnt;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dirty[dlist[i]] = 0;
}

cudaError_t launch_delete_step(sbc_forest* f, int u, int v, const int* d_removed)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(f->d_nwork, 0, 2 * sizeof(int), s)) || (e = cudaMemsetAsync(f->d_nmov, 0, 2 * sizeof(int), s)))
        return e;
    const bool md = f->delete_mode == SBC_DELETE_MOVE_DOWN ||
                    (f->delete_mode == SBC_DELETE_AUTO && f->nv >= kMoveDownMinVertices);
    k_classify_delete<<<(int)((f->nk * 32 + 255) / 256), 256, 0, s>>>(f->d_dist, f->nv, (int)f->nk, g->dev(), u, v,
                                                                      d_removed, f->d_dirty, f->d_worklist,
                                                                      f->d_nwork, f->d_mov, f->d_nmov, md ? 1 : 0,
                                                                      f->d_counters);
    if ((e = cudaGetLastError())) return e;
    // roots that keep a parent: sigma-only update; the others move down (a
    // move-down that outgrows its cap joins the recompute list mov)
    UpdateArgs A;
    A.f = forest_slot(f, 0);
    A.scr = f->scratch();
    A.all_visible = 1;
    A.del_u = u;
    A.del_v = v;
    A.mov = f->d_mov;
    A.nmov = f->d_nmov;
    A.worklist = f->d_worklist;
    A.nwork = f->d_nwork;
    A.work_counter = f->d_counter;
    A.counters = f->d_counters;
    k_delete<512, 1, 4><<<(int)std::min<int64_t>(f->workers, f->nk), 512, 0, s>>>(A);
    if ((e = cudaGetLastError())) return e;
    // the others: their dependencies out of BC now (their state is still that
    // of the graph before this deletion), recomputed at the end of the batch
    const dim3 grid((unsigned)std::min<int64_t>((f->nv + 255) / 256, 64), (unsigned)std::min<int64_t>(f->nk, 4096));
    k_bc_rows<<<grid, 256, 0, s>>>(f->d_delta, f->d_roots, f->d_mov, f->d_nmov, f->nv, f->d_bc, -1.0);
    if ((e = cudaGetLastError())) return e;
    k_mark_dirty<<<(int)std::min<int64_t>((f->nk + 255) / 256, 64), 256, 0, s>>>(f->d_mov, f->d_nmov, f->d_dirty,
                                                                                   f->d_dlist, f->d_dcnt);
    return cudaGetLastError();
}

cudaError_t launch_delete_finish(sbc_forest* f)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    cudaError_t e;
    int n = 0;
    if ((e = cudaMemcpyAsync(&n, f->d_dcnt, sizeof(int), cudaMemcpyDeviceToHost, s)) || (e = cudaStreamSynchronize(s)))
        return e;
    if (n == 0) return cudaSuccess;
    // a few roots of a large graph: one at a time by the whole GPU (a CTA
    // would walk the whole graph alone); otherwise a CTA per root
    if (n <= kWideRecompute && f->nv >= kWideRecomputeMinVertices) {
        std::vector<int> rows(n);
        if ((e = cudaMemcpyAsync(rows.data(), f->d_dlist, sizeof(int) * n, cudaMemcpyDeviceToHost, s)) ||
            (e = cudaStreamSynchronize(s)))
            return e;
        if ((e = recompute_roots_wide(f, rows, f->d_dlist))) return e;
    } else if ((e = launch_static_list(f, f->d_dlist, f->d_dcnt))) {
        return e;
    }
    const dim3 grid((unsigned)std::min<int64_t>((f->nv + 255) / 256, 64), (unsigned)std::min<int64_t>(f->nk, 4096));
    k_bc_rows<<<grid, 256, 0, s>>>(f->d_delta, f->d_roots, f->d_dlist, f->d_dcnt, f->nv, f->d_bc, 1.0);
    if ((e = cudaGetLastError())) return e;
    if ((e = launch_dist2_rows(f, f->d_dlist, f->d_dcnt))) return e;
    if ((e = launch_level_hist_list(f, f->d_dlist, f->d_dcnt))) return e;
    if ((e = launch_roster_build_list(f, f->d_dlist, f->d_dcnt))) return e;
    k_clear_dirty<<<(int)std::min<int64_t>((f->nk + 255) / 256, 64), 256, 0, s>>>(f->d_dlist, f->d_dcnt, f->d_dirty);
    if ((e = cudaGetLastError())) return e;
    return cudaMemsetAsync(f->d_dcnt, 0, sizeof(int), s);
}

// Launch shapes of k_delete_batch: the one with the forest's update shape's
// threads per CTA (its worker scratch then fits: the grid is the forest's
// worker count at most, and a CTA only indexes its own worker slot).
template <int NT, int MINB, int ILP>
void launch_delete_shape(const UpdateArgs& A, int grid, cudaStream_t s)
{
    k_delete_batch<NT, MINB, ILP><<<grid, NT, 0, s>>>(A);
}

struct DeleteShape {
    int threads;
    void (*launch)(const UpdateArgs&, int, cudaStream_t);
};
static const DeleteShape kDeleteShapes[] = {
    {1024, launch_delete_shape<1024, 1, 8>},
    {512, launch_delete_shape<512, 2, 4>},
    {256, launch_delete_shape<256, 4, 4>},
    {128, launch_delete_shape<128, 8, 2>},
};

cudaError_t launch_delete_batch(sbc_forest* f, int n)
{
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(f->d_nwork, 0, 2 * sizeof(int), s))) return e;
    const int32_t* iu = g->d_ins;
    const int32_t* iv = g->d_ins + g->ins_capacity;
    const int32_t* code = g->d_ins + 2 * g->ins_capacity;
    k_classify_delete_batch<<<(int)((f->nk * 32 + 255) / 256), 256, 0, s>>>(f->d_dist, f->nv, (int)f->nk, n, iu, iv,
                                                                            code, f->d_worklist, f->d_nwork);
    if ((e = cudaGetLastError())) return e;
    UpdateArgs A;
    A.f = forest_slot(f, n);
    A.scr = f->scratch();
    A.all_visible = 1;
    A.del_u = A.del_v = 0;
    A.mov = A.nmov = nullptr;
    A.move_down = (f->delete_mode == SBC_DELETE_MOVE_DOWN ||
                   (f->delete_mode == SBC_DELETE_AUTO && f->nv >= kMoveDownMinVertices)) ? 1 : 0;
    A.dirty = f->d_dirty;
    A.dlist = f->d_dlist;
    A.dcnt = f->d_dcnt;
    A.worklist = f->d_worklist;
    A.nwork = f->d_nwork;
    A.work_counter = f->d_counter;
    A.counters = f->d_counters;
    const int want = kVariants[f->variant].threads;
    const DeleteShape* shape = &kDeleteShapes[3];
    for (const DeleteShape& d : kDeleteShapes)
        if (d.threads <= want) {
            shape = &d;
            break;
        }
    shape->launch(A, (int)std::min<int64_t>(f->workers, f->nk), s);
    return cudaGetLastError();
}

cudaError_t launch_delete(sbc_forest* f, int u, int v, const int* d_removed)
{
    cudaError_t e = launch_delete_step(f, u, v, d_removed);
    if (e) return e;
    return launch_delete_finish(f);
}

}  // namespace sbc
