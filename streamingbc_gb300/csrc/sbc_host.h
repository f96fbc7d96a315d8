// Host-side objects behind the C-ABI (include/sbc_gb300.h).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <vector>
#include "sbc_internal.cuh"

#define SBC_NCOUNTERS 5

namespace sbc {

enum ProfKernel { PROF_STATIC = 0, PROF_APPEND, PROF_CLASSIFY, PROF_UPDATE, PROF_BATCH, PROF_COUNT };

}  // namespace sbc

struct sbc_forest;

namespace sbc {
// Cost model: an FP32 MLP 8 -> 64 -> 64 -> 1 (ReLU) predicting log(1 + touched
// vertices) of one (insertion, root) job.  Parameter layout in floats:
constexpr int kIn = 8, kH = 64;
constexpr int OFF_W1 = 0;                  // [kIn][kH]
constexpr int OFF_B1 = OFF_W1 + kIn * kH;  // [kH]
constexpr int OFF_W2 = OFF_B1 + kH;        // [kH][kH]
constexpr int OFF_B2 = OFF_W2 + kH * kH;   // [kH]
constexpr int OFF_W3 = OFF_B2 + kH;        // [kH]
constexpr int OFF_B3 = OFF_W3 + kH;        // [1]
constexpr int kTrainParams = OFF_B3 + 1;   // trained parameters
constexpr int OFF_MU = kTrainParams;       // [kIn] feature means
constexpr int OFF_ISD = OFF_MU + kIn;      // [kIn] inverse feature standard deviations
constexpr int kModelParams = OFF_ISD + kIn;
constexpr int kCostBuckets = 256;          // ordering buckets: 8 per doubling of predicted cost
}  // namespace sbc

// Training data, parameters and per-batch buffers of a forest's cost model.
struct CostModel {
    bool logging = false;   // log (features, touched vertices) of every job of later batches
    bool trained = false;
    int64_t capacity = 0;   // training samples the log holds
    int adam_t = 0;
    float* d_params = nullptr;  // [kModelParams]
    float* d_m = nullptr;       // Adam moments [kTrainParams]
    float* d_v = nullptr;
    float* d_grad = nullptr;    // [kTrainParams]
    float* d_x = nullptr;       // [capacity][kIn] features
    float* d_y = nullptr;       // [capacity] log(1 + touched vertices)
    unsigned long long* d_n = nullptr;  // samples appended (may exceed capacity; the excess is dropped)
    double* d_sums = nullptr;   // [32] reduction accumulators
    int64_t log_ins = 0;        // batch size the two per-batch buffers hold
    float* d_feat = nullptr;    // [nk][log_ins][kIn] features of the batch's (root, insertion) pairs
    int32_t* d_cost_log = nullptr;  // [nk][log_ins] touched vertices, -1 where no job ran
    float* d_root_cost = nullptr;   // [nk] predicted touched vertices of the batch, -1 if culled
    int* d_buckets = nullptr;       // [kCostBuckets]
};

// Scratch of a set of persistent update/static workers, each sized for nv
// vertices: step/state word, queues and level offsets (int32), diffPath
// (int64), delta accumulator (fp64) and one bitmap bit per vertex.  Zeroed on
// allocation; every job leaves what it touched zeroed again.
struct WorkerScratch {
    int64_t workers = 0, nv = 0;
    int32_t* st = nullptr;
    int64_t* dp = nullptr;
    double* acc = nullptr;
    int32_t* qd = nullptr;
    int32_t* qa = nullptr;
    int32_t* qs = nullptr;
    int32_t* lvl = nullptr;
    uint32_t* bits = nullptr;

    static size_t per_worker(int64_t nv) { return (size_t)nv * 36 + sbc::bitmap_words(nv) * 4 + 16; }
    size_t bytes() const
    {
        return (size_t)workers * ((size_t)nv * 36 + (size_t)8 + sbc::bitmap_words(nv) * 4);
    }
    void release()
    {
        for (void* p : {(void*)st, (void*)dp, (void*)acc, (void*)qd, (void*)qa, (void*)qs, (void*)lvl, (void*)bits})
            if (p) cudaFree(p);
        st = qd = qa = qs = lvl = nullptr;
        dp = nullptr;
        acc = nullptr;
        bits = nullptr;
        workers = 0;
    }
    cudaError_t alloc(int64_t w, int64_t n, cudaStream_t s)
    {
        release();
        const size_t sc = (size_t)w * (size_t)n, words = (size_t)w * sbc::bitmap_words(n);
        cudaError_t e;
        if ((e = cudaMalloc(&st, sc * 4)) || (e = cudaMalloc(&dp, sc * 8)) || (e = cudaMalloc(&acc, sc * 8)) ||
            (e = cudaMalloc(&qd, sc * 4)) || (e = cudaMalloc(&qa, sc * 4)) || (e = cudaMalloc(&qs, sc * 4)) ||
            (e = cudaMalloc(&lvl, (size_t)w * (size_t)(n + 2) * 4)) || (e = cudaMalloc(&bits, words * 4))) {
            release();
            return e;
        }
        workers = w;
        nv = n;
        if ((e = cudaMemsetAsync(st, 0, sc * 4, s)) || (e = cudaMemsetAsync(dp, 0, sc * 8, s)) ||
            (e = cudaMemsetAsync(acc, 0, sc * 8, s)) || (e = cudaMemsetAsync(bits, 0, words * 4, s)))
            return e;
        return cudaSuccess;
    }
    sbc::ScratchBase base() const
    {
        sbc::ScratchBase b;
        b.st = st;
        b.dp = dp;
        b.acc = acc;
        b.qd = qd;
        b.qa = qa;
        b.qs = qs;
        b.lvl = lvl;
        b.bits = bits;
        return b;
    }
};

// Device-resident slack-CSR adjacency (replaces the STINGER edge-block store,
// src/stinger/stinger-internal.h:45-103).  All device work for the graph and
// for forests bound to it runs on `stream`, in order.
struct sbc_graph {
    int device = 0;
    cudaStream_t stream = nullptr;
    int64_t nv = 0;
    int64_t total_cap = 0;
    int64_t* d_row = nullptr;
    int32_t* d_deg = nullptr;
    int32_t* d_deg0 = nullptr;
    int32_t* d_nsort = nullptr;  // leading slots of each vertex stored in sorted order
    int32_t* d_cap = nullptr;
    int32_t* d_col = nullptr;
    int32_t* d_seq = nullptr;
    int* d_err = nullptr;
    // host mirrors used to plan re-packs without reading the device
    std::vector<int64_t> h_row;
    std::vector<int32_t> h_cap;
    std::vector<int64_t> h_deg_ub;  // upper bound of the live degree
    // staging for insertion batches
    int ins_capacity = 0;
    int32_t* d_ins = nullptr;  // [5 * ins_capacity + 1]: u, v, ok, then the append's ranks and misfit flag
    int32_t* h_ins = nullptr;  // pinned [3 * ins_capacity]
    cudaEvent_t staged = nullptr;  // recorded after the last copy out of h_ins
    const int32_t** d_src = nullptr;  // device slot: addresses of the caller's endpoint arrays
    int64_t repacks = 0;
    // forests bound to this graph; destroying the graph detaches them
    std::vector<sbc_forest*> forests;
    bool last_directed = false;  // the staged insertions were appended one direction only

    sbc::DevGraph dev() const
    {
        sbc::DevGraph G;
        G.nv = nv;
        G.row = d_row;
        G.deg = d_deg;
        G.deg0 = d_deg0;
        G.nsort = d_nsort;
        G.col = d_col;
        G.seq = d_seq;
        return G;
    }
};

struct sbc_forest {
    sbc_graph* g = nullptr;  // null once the graph has been destroyed
    int device = 0;
    int64_t nv = 0, nk = 0;
    std::vector<int64_t> h_roots;
    int64_t* d_roots = nullptr;
    int32_t* d_dist = nullptr;
    uint8_t* d_dist8 = nullptr;  // one-byte shadow of d_dist gathered by the walkers
    uint32_t* d_dist2 = nullptr; // [nk][d2_words(nv)] two-bit shadow (dist mod 3) gathered by the update walks
    int64_t* d_sigma = nullptr;
    double* d_delta = nullptr;
    double* d_bc = nullptr;
    bool initialized = false;
    // persistent workers and their scratch
    int sm_count = 0;
    int variant = 0;  // launch shape of the update kernel
    int delete_mode = 0;  // SBC_DELETE_*: lost-parent roots moved down or recomputed
    int64_t workers = 0;      // == ws.workers
    int64_t workers_req = 0;  // worker count the caller asked for (0 = one per resident CTA)
    int groups = 0;           // groups this forest is a member of
    int32_t* d_lvlhist = nullptr;  // [nk][kHistLevels] vertices per level of each root's tree
    int32_t* d_roster = nullptr;   // [nk][kRosterLevels][kRosterCap] small-level members (null: no rosters)
    int32_t* d_roster_n = nullptr;
    int32_t* d_roster_dirty = nullptr;
    // level-2 parent masks (null when they would not fit): [nk][nv] masks,
    // [nk][kL1Max] root neighbours, [nk] their counts, and the roots whose
    // masks must be rebuilt after the current graph change ([nk] flags,
    // [nk] list, [1] count)
    uint32_t* d_l2mask = nullptr;
    int32_t* d_l1cand = nullptr;
    int32_t* d_l1n = nullptr;
    int32_t* d_l2flag = nullptr;
    int32_t* d_l2list = nullptr;
    int32_t* d_l2cnt = nullptr;
    CostModel* model = nullptr;    // allocated by the first cost-model call
    int schedule = 0;              // root order of a batch: 0 static (classify order), 1 cost model
    int64_t state_bytes = 0;
    WorkerScratch ws;
    int* d_worklist = nullptr;
    int* d_mov = nullptr;     // [nk] roots of a deletion left to a recompute (move-down over its cap)
    int* d_nmov = nullptr;    // [2]: their count, work counter
    // roots left for a recompute at the end of a deletion batch: [nk] flags,
    // [nk] list, [1] count
    int* d_dirty = nullptr;
    int* d_dlist = nullptr;
    int* d_dcnt = nullptr;
    int* d_wide = nullptr;    // [3 * kWideRecompute]: BFS lengths and level ranges of the wide recompute
    int* d_res = nullptr;     // [1] result of the last edge removal
    int* d_nwork = nullptr;   // [1]
    int* d_counter = nullptr; // [1]
    // [SBC_NCOUNTERS]: traversed vertices, traversed edges (reference counters),
    // case-1 pairs, case-2 pairs, adjacency slots actually scanned
    unsigned long long* d_counters = nullptr;
    int64_t bytes = 0;
    // Device-input batches replayed from captured CUDA graphs, one per batch
    // size; only the two input copies are re-pointed per call.  A graph is
    // re-captured when the adjacency was re-packed or the staging moved.
    struct CapturedBatch {
        cudaGraphExec_t exec = nullptr;
        int64_t repacks = -1;
        const int32_t* d_ins = nullptr;
    };
    bool use_graphs = true;
    std::vector<std::pair<int, CapturedBatch>> captured;
    // profiling: a ring of CUDA event pairs per kernel kind; pairs are read
    // back only when the ring wraps or the profile is queried, so recording
    // never makes the host wait for the device.
    static constexpr int kRing = 512;
    bool prof = false;
    std::vector<cudaEvent_t> ev_a[sbc::PROF_COUNT];
    std::vector<cudaEvent_t> ev_b[sbc::PROF_COUNT];
    std::vector<char> ev_pending[sbc::PROF_COUNT];
    int ev_next[sbc::PROF_COUNT] = {};
    double prof_ms[sbc::PROF_COUNT] = {};
    int64_t prof_n[sbc::PROF_COUNT] = {};
    cudaEvent_t t0 = nullptr, t1 = nullptr;

    sbc::ScratchBase scratch() const { return ws.base(); }
    cudaError_t prof_init()
    {
        for (int k = 0; k < sbc::PROF_COUNT; ++k) {
            ev_a[k].assign(kRing, nullptr);
            ev_b[k].assign(kRing, nullptr);
            ev_pending[k].assign(kRing, 0);
            for (int i = 0; i < kRing; ++i) {
                cudaError_t e;
                if ((e = cudaEventCreate(&ev_a[k][i])) || (e = cudaEventCreate(&ev_b[k][i]))) return e;
            }
        }
        return cudaSuccess;
    }
    void prof_release()
    {
        for (int k = 0; k < sbc::PROF_COUNT; ++k) {
            for (auto e : ev_a[k])
                if (e) cudaEventDestroy(e);
            for (auto e : ev_b[k])
                if (e) cudaEventDestroy(e);
            ev_a[k].clear();
            ev_b[k].clear();
        }
    }
    void prof_collect_slot(int k, int i)
    {
        if (!ev_pending[k][i]) return;
        float ms = 0.f;
        cudaEventSynchronize(ev_b[k][i]);
        cudaEventElapsedTime(&ms, ev_a[k][i], ev_b[k][i]);
        prof_ms[k] += ms;
        prof_n[k] += 1;
        ev_pending[k][i] = 0;
    }
    void prof_collect(int k)
    {
        for (int i = 0; i < (int)ev_pending[k].size(); ++i) prof_collect_slot(k, i);
    }
    void prof_begin(int k)
    {
        if (!prof) return;
        const int i = ev_next[k];
        prof_collect_slot(k, i);
        cudaEventRecord(ev_a[k][i], g->stream);
    }
    void prof_end(int k)
    {
        if (!prof) return;
        const int i = ev_next[k];
        cudaEventRecord(ev_b[k][i], g->stream);
        ev_pending[k][i] = 1;
        ev_next[k] = (i + 1) % kRing;
    }
};

// Forests over different graphs updated together: one append, classify and
// persistent update launch per batch on the group's own stream, with the
// group's own worker scratch (stride: the largest member's vertex count).
// members[s] is slot s (largest roots x vertices first); order[s] is the
// index the caller gave that member.
struct sbc_group {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<sbc_forest*> members;
    std::vector<int> order;
    int sm_count = 0;
    int variant = 0;
    int64_t nv_max = 0, total_roots = 0;
    WorkerScratch ws;
    uint32_t* d_worklist = nullptr;
    int* d_nwork = nullptr;  // [2]: nwork, work counter
    unsigned long long* d_counters = nullptr;  // [SBC_NCOUNTERS]
    cudaEvent_t ev = nullptr;                  // stream hand-off
    cudaEvent_t t0 = nullptr, t1 = nullptr;    // device time of the last batch
    double* h_bc = nullptr;                    // pinned staging of every member's BC
    int64_t h_bc_cap = 0;
    int* d_errs = nullptr;  // [kMaxGroup]: each slot's slack error flag after a batch (the seal gathers them)
    int* h_errs = nullptr;  // pinned copy
};

namespace sbc {
// Most forests (and graphs) one group launch takes.
constexpr int kMaxGroup = 64;

// One graph's staged batch as the group append and seal kernels see it.
struct GraphBatchSlot {
    int64_t nv;
    const int64_t* row;
    int32_t* deg;
    int32_t* deg0;
    int32_t* nsort;
    const int32_t* cap;
    int32_t* col;
    int32_t* seq;
    const int32_t* iu;
    const int32_t* iv;
    int32_t* ok;
    int* err;
    int n;
};
struct GraphBatchSlots {
    GraphBatchSlot slot[kMaxGroup];
    int count;
    int* errs = nullptr;  // when set, the seal copies slot s's error flag to errs[s]
};
GraphBatchSlot graph_batch_slot(sbc_graph* g, int n);
cudaError_t launch_append_group(const GraphBatchSlots& S, cudaStream_t s);
cudaError_t launch_seal_group(const GraphBatchSlots& S, cudaStream_t s);

// Device view of forest f with the n insertions staged in its graph.
inline ForestSlot forest_slot(const sbc_forest* f, int n)
{
    const sbc_graph* g = f->g;
    ForestSlot s;
    s.G = g->dev();
    s.roots = f->d_roots;
    s.dist = f->d_dist;
    s.dist8 = f->d_dist8;
    s.dist2 = f->d_dist2;
    s.sigma = f->d_sigma;
    s.delta = f->d_delta;
    s.bc = f->d_bc;
    s.ins_u = g->d_ins;
    s.ins_v = g->d_ins + g->ins_capacity;
    s.ins_ok = g->d_ins + 2 * g->ins_capacity;
    s.nins = n;
    s.nk = (int)f->nk;
    s.lvlhist = f->d_lvlhist;
    s.cost_log = nullptr;
    s.roster = f->d_roster;
    s.roster_n = f->d_roster_n;
    s.roster_dirty = f->d_roster_dirty;
    s.l2mask = f->d_l2mask;
    s.l1cand = f->d_l1cand;
    s.l1n = f->d_l1n;
    return s;
}

int static_workers_per_sm();
int update_variant_count();
int update_default_variant();
int update_variant_threads(int v);
int update_workers_per_sm(int v);
// Sets the calling thread's sbc_last_error() message and returns code.
int report_error(int code, const char* fmt, ...);
// Scatters the caller's host CSR into the device slack layout (d_row, d_deg
// already set; deg = the live degrees) and sorts every vertex's list on the
// device.  Synchronous on s.
cudaError_t build_adjacency(int64_t nv, const int64_t* off, const int64_t* adj, const int64_t* d_row,
                            const int32_t* d_deg, const std::vector<int32_t>& deg, int32_t* d_col, int sm_count,
                            cudaStream_t s);
cudaError_t launch_static(sbc_forest* f);
// Classify + cull + update for insertions already staged in g->d_ins
// (u, v, ok rows).  `all_visible` ignores the per-slot sequence numbers.
cudaError_t launch_update(sbc_forest* f, int n, bool all_visible);
cudaError_t launch_append(sbc_graph* g, int n, bool directed);
// Record the addresses of device-resident endpoint arrays (one-thread kernel),
// then copy them into the staging rows (the part a batch graph replays).
cudaError_t launch_set_src(sbc_graph* g, const int32_t* d_u, const int32_t* d_v);
cudaError_t launch_stage(sbc_graph* g, int n);
cudaError_t launch_seal(sbc_graph* g, int n);
cudaError_t launch_repack(sbc_graph* g, const int64_t* d_new_row, int32_t* d_new_col, int32_t* d_new_seq);
// Edge removal (both directions unless directed); *d_res = 1 removed, 0 absent, -1 invalid.
cudaError_t launch_remove(sbc_graph* g, int u, int v, bool directed, int* d_res);
// Update for the deletion of (u, v), already removed from the adjacency
// (*d_removed must be 1, else nothing is done): roots that keep a parent of the
// deeper endpoint get the sigma-decrease descent and ascent; the others move
// down or are recomputed from scratch (SBC_DELETE_*), a recomputed root's old
// dependencies taken out of BC first.
// launch_delete_step: the update of one deletion, recomputes left for
// launch_delete_finish, which recomputes the listed roots once on the graph as
// it then stands and puts their rows back.
cudaError_t launch_delete_step(sbc_forest* f, int u, int v, const int* d_removed);
cudaError_t launch_delete_finish(sbc_forest* f);
cudaError_t launch_delete(sbc_forest* f, int u, int v, const int* d_removed);
// Every root through the n deletions marked in g's staging (launch_mark_removed),
// in one persistent launch; dirty roots are left for launch_delete_finish.
cudaError_t launch_delete_batch(sbc_forest* f, int n);
// Static recompute of the roots listed (device list and count) or, with a
// null list, of all roots.
cudaError_t launch_static_list(sbc_forest* f, const int* d_list, const int* d_nlist);
// Whole-GPU recompute of the listed root rows (rows on the host, d_rows the
// same list on the device), all of them level by level together
// (level-synchronous, synchronous); used by deletions on graphs of at least
// kWideRecomputeMinVertices vertices for up to kWideRecompute roots, the
// static kernel otherwise.
cudaError_t recompute_roots_wide(sbc_forest* f, const std::vector<int>& rows, const int* d_rows);
constexpr int kWideRecompute = 64;
constexpr int64_t kWideRecomputeMinVertices = 32768;
cudaError_t launch_level_hist_list(sbc_forest* f, const int* d_list, const int* d_nlist);
// Two-bit rows of every root (or the listed roots) derived from their dist rows.
cudaError_t launch_dist2_rows(sbc_forest* f, const int* d_list, const int* d_nlist);
// Level-2 parent masks of every root (after static init or a restore).
cudaError_t launch_l2mask_build_all(sbc_forest* f);
// Masks of every forest of g after the n insertions staged in g were appended
// (directed: only the u -> v slots), and after the removal of (u, v) when
// *d_removed (directed: the u -> v slot only).
cudaError_t launch_l2mask_insert(sbc_graph* g, int n, bool directed);
cudaError_t launch_l2mask_insert_forest(sbc_forest* f, int n, bool directed, cudaStream_t s);
// The same for nf forests (counts[j] insertions staged on fs[j]'s graph), one
// launch per step for up to kMaxGroup forests.
cudaError_t launch_l2mask_insert_forests(sbc_forest* const* fs, const int* counts, int nf, bool directed,
                                        cudaStream_t s);
cudaError_t launch_l2mask_remove(sbc_graph* g, int u, int v, bool directed, const int* d_removed);
// ... and after the n removals staged in g (undirected; codes in the staging's
// third row), once their slots are compacted.
cudaError_t launch_l2mask_remove_batch(sbc_graph* g, int n);
// Batched deletions of the n edges staged in g: removal marks in order
// (codes into the staging's third row), and after the update the compaction
// of the marked slots (and the masks' upkeep).
cudaError_t launch_mark_removed(sbc_graph* g, int n);
// Largest batch appended a warp per insertion (larger ones: one warp in order).
constexpr int kParallelAppendMax = 8192;
cudaError_t launch_compact_removed(sbc_graph* g, int n);
cudaError_t launch_roster_build_list(sbc_forest* f, const int* d_list, const int* d_nlist);
// Cost model and schedule (sbc_model.cu).
cudaError_t launch_level_hist(sbc_forest* f);
// Rosters of every root from its distances (after static init), and the
// compaction of rosters that hold stale entries (after each batch).
cudaError_t launch_roster_build(sbc_forest* f);
cudaError_t launch_roster_compact(sbc_forest* f, cudaStream_t s);
cudaError_t launch_roster_compact_forests(sbc_forest* const* fs, int nf, cudaStream_t s);
// Deletions move lost-parent roots down (rather than recompute them) on graphs
// of at least this many vertices under SBC_DELETE_AUTO.
constexpr int64_t kMoveDownMinVertices = 32768;
// Before the update of a batch of n: features of every active (root,
// insertion) pair into the log buffers (when logging) and, under the model
// schedule, the worklist ordered by predicted cost (longest first);
// returns whether it built the worklist.
cudaError_t launch_schedule(sbc_forest* f, int n, bool* built_worklist);
// After the update: the batch's logged (features, cost) pairs into the training set.
cudaError_t launch_log_append(sbc_forest* f, int n);
cudaError_t launch_moments(sbc_forest* f, int64_t n);
// Mean-squared-error gradient of samples at positions [base, base+count) of
// the permutation j -> (j * mul + add) % n of (d_x, d_y), added into d_grad;
// predictions into d_pred (may be null).
cudaError_t launch_grad(const float* d_params, float* d_grad, const float* d_x, const float* d_y, int64_t base,
                        int64_t count, int64_t n, int64_t mul, int64_t add, float* d_pred, cudaStream_t s);
// launch_grad over the forest's training set, then one Adam step.
cudaError_t launch_train_step(sbc_forest* f, int64_t base, int64_t count, int64_t n, int64_t mul, int64_t add, float lr);
cudaError_t launch_eval(sbc_forest* f, int64_t lo, int64_t hi, float ymean);
cudaError_t launch_predict(const float* d_params, const float* d_x, int64_t n, float* d_out, cudaStream_t s);
int group_variant_count();
int group_workers_per_sm(int v);
// Append, classify + update, and seal (the steps selected) for the counts[s]
// insertions staged in each member s's graph, on the group's stream.
enum GroupSteps : unsigned { GROUP_APPEND = 1, GROUP_UPDATE = 2, GROUP_SEAL = 4, GROUP_ALL = 7 };
cudaError_t launch_group_update(sbc_group* G, const int* counts, unsigned steps);
}  // namespace sbc
