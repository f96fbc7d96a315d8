// Multi-forest batches: many forests, each over its own graph, updated by one
// classify launch and one persistent update launch per batch.
//
// The reference updates one forest per insertEdgeStreamingBC call
// (src/streamingbc.c:88-226); a caller with many small graphs pays one full
// pass of launches per graph and leaves most SMs idle on each.  Here a group
// stages every member's insertions, appends them all in one launch (one warp
// per graph, k_append_group), culls roots of all members in one classify
// launch, and runs one persistent update launch whose work items are
// (member, root) pairs drawn from a single queue, so large and small graphs
// share the SMs.  Each item is processed by exactly the per-root code of the
// single-forest kernel (process_root), so results are those of updating the
// members one by one.  Members occupy slots largest first (roots x vertices),
// which puts the longest items at the front of the queue.
#include <algorithm>
#include <vector>
#include "sbc_host.h"
#include "sbc_update_job.cuh"

namespace sbc {

// worklist entry: slot << kSlotShift | root
constexpr int kSlotShift = 25;
constexpr uint32_t kRootMask = (1u << kSlotShift) - 1u;

struct GroupUpdateArgs {
    ForestSlot slot[kMaxGroup];
    int root_base[kMaxGroup + 1];  // prefix sums of the members' root counts
    int nslots;
    ScratchBase scr;
    int64_t scr_nv;  // per-worker scratch stride: the largest member's vertex count
    uint32_t* worklist;
    int* nwork;
    int* work_counter;
    unsigned long long* counters;
};

// One thread per (member, root): the pair joins the batch's worklist iff some
// live insertion of that member's batch joins two different levels of the
// root's tree (as k_classify does for one forest).
__global__ void k_classify_group(const __grid_constant__ GroupUpdateArgs A)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.root_base[A.nslots]) return;
    int lo = 0, hi = A.nslots - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (A.root_base[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    const ForestSlot& P = A.slot[lo];
    const int r = i - A.root_base[lo];
    const int32_t* D = P.dist + (size_t)r * P.G.nv;
    bool active = false;
    for (int k = 0; k < P.nins && !active; ++k)
        if (P.ins_ok[k] > 0 && D[P.ins_u[k]] != D[P.ins_v[k]]) active = true;
    if (active) A.worklist[atomicAdd(A.nwork, 1)] = ((uint32_t)lo << kSlotShift) | (uint32_t)r;
}

template <int NT, int MINB, int ILP>
__global__ void __launch_bounds__(NT, MINB) k_update_group(const __grid_constant__ GroupUpdateArgs A)
{
    __shared__ UpdSmem<NT> sm;
    const Scratch W = A.scr.of(blockIdx.x, A.scr_nv);
    const int nwork = *A.nwork;
    reset_counters<NT>(sm);
    for (;;) {
        if (threadIdx.x == 0) sm.item = atomicAdd(A.work_counter, 1);
        __syncthreads();
        const int item = sm.item;
        __syncthreads();
        if (item >= nwork) break;
        const uint32_t e = A.worklist[item];
        process_root<NT, ILP>(A.slot[e >> kSlotShift], sm, W, (int)(e & kRootMask), false);
    }
    flush_counters<NT>(sm, A.counters);
}

template <int NT, int MINB, int ILP>
void launch_group_variant(const GroupUpdateArgs& A, int grid, cudaStream_t s)
{
    k_update_group<NT, MINB, ILP><<<grid, NT, 0, s>>>(A);
}

template <int NT, int MINB, int ILP>
int occupancy_group_variant()
{
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_update_group<NT, MINB, ILP>, NT, 0);
    return n;
}

struct GroupVariant {
    int threads, min_blocks, ilp;
    void (*launch)(const GroupUpdateArgs&, int, cudaStream_t);
    int (*occupancy)();
};

// Same shapes, in the same order, as the single-forest update kernel's table.
static const GroupVariant kGroupVariants[] = {
    {256, 4, 4, launch_group_variant<256, 4, 4>, occupancy_group_variant<256, 4, 4>},
    {256, 5, 4, launch_group_variant<256, 5, 4>, occupancy_group_variant<256, 5, 4>},
    {256, 6, 4, launch_group_variant<256, 6, 4>, occupancy_group_variant<256, 6, 4>},
    {128, 8, 4, launch_group_variant<128, 8, 4>, occupancy_group_variant<128, 8, 4>},
    {128, 10, 4, launch_group_variant<128, 10, 4>, occupancy_group_variant<128, 10, 4>},
    {512, 2, 4, launch_group_variant<512, 2, 4>, occupancy_group_variant<512, 2, 4>},
    {512, 1, 4, launch_group_variant<512, 1, 4>, occupancy_group_variant<512, 1, 4>},
    {1024, 1, 4, launch_group_variant<1024, 1, 4>, occupancy_group_variant<1024, 1, 4>},
    {64, 16, 4, launch_group_variant<64, 16, 4>, occupancy_group_variant<64, 16, 4>},
    {32, 32, 4, launch_group_variant<32, 32, 4>, occupancy_group_variant<32, 32, 4>},
    // deeper (8) or shallower (2) gather pipelines per thread
    {1024, 1, 8, launch_group_variant<1024, 1, 8>, occupancy_group_variant<1024, 1, 8>},
    {512, 2, 8, launch_group_variant<512, 2, 8>, occupancy_group_variant<512, 2, 8>},
    {128, 8, 2, launch_group_variant<128, 8, 2>, occupancy_group_variant<128, 8, 2>},
    {256, 4, 2, launch_group_variant<256, 4, 2>, occupancy_group_variant<256, 4, 2>},
};
constexpr int kNumGroupVariants = sizeof(kGroupVariants) / sizeof(kGroupVariants[0]);

int group_variant_count() { return kNumGroupVariants; }
int group_workers_per_sm(int v) { return kGroupVariants[v].occupancy(); }

cudaError_t launch_group_update(sbc_group* G, const int* counts, unsigned steps)
{
    cudaStream_t s = G->stream;
    cudaError_t e;
    const int ns = (int)G->members.size();
    GraphBatchSlots B;
    B.count = ns;
    B.errs = G->d_errs;
    GroupUpdateArgs A;
    A.nslots = ns;
    A.root_base[0] = 0;
    for (int i = 0; i < ns; ++i) {
        sbc_forest* f = G->members[i];
        B.slot[i] = graph_batch_slot(f->g, counts[i]);
        A.slot[i] = forest_slot(f, counts[i]);
        A.root_base[i + 1] = A.root_base[i] + (int)f->nk;
    }
    A.scr = G->ws.base();
    A.scr_nv = G->ws.nv;
    A.worklist = G->d_worklist;
    A.nwork = G->d_nwork;
    A.work_counter = G->d_nwork + 1;
    A.counters = G->d_counters;
    if ((steps & GROUP_APPEND) && (e = launch_append_group(B, s))) return e;
    if (steps & GROUP_UPDATE) {
        if ((e = cudaMemsetAsync(G->d_nwork, 0, 2 * sizeof(int), s))) return e;
        const int total = A.root_base[ns];
        k_classify_group<<<(total + 255) / 256, 256, 0, s>>>(A);
        if ((e = cudaGetLastError())) return e;
        const int grid = (int)std::min<int64_t>(G->ws.workers, total);
        kGroupVariants[G->variant].launch(A, grid, s);
        if ((e = cudaGetLastError())) return e;
        if ((e = launch_roster_compact_forests(G->members.data(), ns, s))) return e;
    }
    if (steps & GROUP_SEAL) {
        if ((e = launch_seal_group(B, s))) return e;
        // level-2 masks of every forest on the members' graphs
        std::vector<sbc_forest*> fs;
        std::vector<int> fc;
        for (int i = 0; i < ns; ++i)
            for (sbc_forest* f : G->members[i]->g->forests) {
                if (std::find(fs.begin(), fs.end(), f) != fs.end()) continue;
                fs.push_back(f);
                fc.push_back(counts[i]);
            }
        if ((e = launch_l2mask_insert_forests(fs.data(), fc.data(), (int)fs.size(), false, s))) return e;
    }
    return cudaSuccess;
}

}  // namespace sbc
