// C-ABI of libsbc_gb300.so: sbc_* entry points (include/sbc_gb300.h), the
// drop-in streamingbc.h surface of the reference and the STINGER shim.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <random>
#include <unordered_map>
#include <vector>

#include "sbc_gb300.h"
#include "streamingbc.h"
#include "sbc_host.h"

namespace {

thread_local std::string t_err;
thread_local int t_device = -1;

int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* where)
{
    return fail(e == cudaErrorMemoryAllocation ? SBC_ERR_NOMEM : SBC_ERR_CUDA, "%s: %s", where,
                cudaGetErrorString(e));
}

#define CK(call)                                         \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

template <class T>
cudaError_t dev_alloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

template <class T>
void dev_free(T*& p)
{
    if (p) cudaFree(p);
    p = nullptr;
}

int use_device(int dev) { return cudaSetDevice(dev) == cudaSuccess ? SBC_OK : fail(SBC_ERR_CUDA, "cudaSetDevice(%d) failed", dev); }

int current_device()
{
    if (t_device >= 0) return t_device;
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

// Slack policy: room for max(4, deg/8) more neighbours per vertex.
int32_t slack_cap(int64_t live)
{
    int64_t c = live + std::max<int64_t>(4, live / 8);
    return (int32_t)std::min<int64_t>(c, INT32_MAX - 1);
}

int ensure_staging(sbc_graph* g, int64_t n)
{
    if (n <= g->ins_capacity) return SBC_OK;
    int cap = (int)std::max<int64_t>(n, 64);
    CK(cudaStreamSynchronize(g->stream));  // queued batches may still read the old staging
    if (g->d_ins) cudaFree(g->d_ins);
    if (g->h_ins) cudaFreeHost(g->h_ins);
    g->d_ins = nullptr;
    g->h_ins = nullptr;
    CK(dev_alloc(&g->d_ins, (size_t)5 * cap + 1));  // u, v, codes, two rank rows and a flag (launch_append)
    CK(cudaMallocHost((void**)&g->h_ins, sizeof(int32_t) * 3 * (size_t)cap));
    g->ins_capacity = cap;
    return SBC_OK;
}

// Re-pack the adjacency so that every vertex has room for need[v] more slots.
int repack(sbc_graph* g, const std::unordered_map<int64_t, int64_t>& need)
{
    CK(cudaStreamSynchronize(g->stream));
    std::vector<int32_t> deg(g->nv);
    if (g->nv) CK(cudaMemcpy(deg.data(), g->d_deg, sizeof(int32_t) * g->nv, cudaMemcpyDeviceToHost));
    std::vector<int64_t> row(g->nv + 1);
    std::vector<int32_t> cap(g->nv);
    int64_t total = 0;
    for (int64_t v = 0; v < g->nv; ++v) {
        auto it = need.find(v);
        int64_t want = deg[v] + (it == need.end() ? 0 : it->second);
        int32_t c = std::max<int32_t>(g->h_cap[v], slack_cap(want));
        if (it != need.end()) c = std::max<int32_t>(c, slack_cap(want + want / 4));
        row[v] = total;
        cap[v] = c;
        total += c;
    }
    row[g->nv] = total;
    int64_t* d_row = nullptr;
    int32_t *d_col = nullptr, *d_seq = nullptr;
    cudaError_t e;
    if ((e = dev_alloc(&d_row, g->nv + 1)) || (e = dev_alloc(&d_col, total)) || (e = dev_alloc(&d_seq, total))) {
        dev_free(d_row);
        dev_free(d_col);
        dev_free(d_seq);
        return cuda_fail(e, "repack allocation");
    }
    CK(cudaMemcpyAsync(d_row, row.data(), sizeof(int64_t) * (g->nv + 1), cudaMemcpyHostToDevice, g->stream));
    CK(sbc::launch_repack(g, d_row, d_col, d_seq));
    CK(cudaMemcpyAsync(g->d_cap, cap.data(), sizeof(int32_t) * g->nv, cudaMemcpyHostToDevice, g->stream));
    CK(cudaMemcpyAsync(g->d_deg0, g->d_deg, sizeof(int32_t) * g->nv, cudaMemcpyDeviceToDevice, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    dev_free(g->d_row);
    dev_free(g->d_col);
    dev_free(g->d_seq);
    g->d_row = d_row;
    g->d_col = d_col;
    g->d_seq = d_seq;
    g->total_cap = total;
    g->h_row = row;
    g->h_cap = cap;
    for (int64_t v = 0; v < g->nv; ++v) g->h_deg_ub[v] = deg[v];
    g->repacks++;
    return SBC_OK;
}

// Make sure the n undirected (or directed) insertions fit in the slack;
// counts them into the host degree upper bound.
int plan_capacity(sbc_graph* g, int64_t n, const int64_t* u, const int64_t* v, bool directed)
{
    std::unordered_map<int64_t, int64_t> need;
    bool over = false;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t a = u[i], b = v[i];
        if (a == b || a < 0 || b < 0 || a >= g->nv || b >= g->nv) continue;
        int64_t na = ++need[a];
        if (g->h_deg_ub[a] + na > g->h_cap[a]) over = true;
        if (!directed) {
            int64_t nb = ++need[b];
            if (g->h_deg_ub[b] + nb > g->h_cap[b]) over = true;
        }
    }
    if (over) {
        int rc = repack(g, need);
        if (rc) return rc;
    }
    for (auto& kv : need) g->h_deg_ub[kv.first] += kv.second;
    return SBC_OK;
}

int stage_host(sbc_graph* g, int64_t n, const int64_t* u, const int64_t* v, bool set_ok)
{
    int rc = ensure_staging(g, n);
    if (rc) return rc;
    const int cap = g->ins_capacity;
    if (g->staged) CK(cudaEventSynchronize(g->staged));  // the previous batch's copies out of h_ins are done
    int32_t* hu = g->h_ins;
    int32_t* hv = g->h_ins + cap;
    int32_t* hok = g->h_ins + 2 * cap;
    for (int64_t i = 0; i < n; ++i) {
        const bool valid = u[i] >= 0 && v[i] >= 0 && u[i] < g->nv && v[i] < g->nv && u[i] != v[i];
        hu[i] = valid ? (int32_t)u[i] : 0;
        hv[i] = valid ? (int32_t)v[i] : 0;
        hok[i] = valid ? 1 : -1;
        if (!valid) {
            // keep ids in range so the append kernel rejects cleanly as a loop
            hu[i] = -1;
            hv[i] = -1;
        }
    }
    CK(cudaMemcpyAsync(g->d_ins, hu, sizeof(int32_t) * n, cudaMemcpyHostToDevice, g->stream));
    CK(cudaMemcpyAsync(g->d_ins + cap, hv, sizeof(int32_t) * n, cudaMemcpyHostToDevice, g->stream));
    if (set_ok) CK(cudaMemcpyAsync(g->d_ins + 2 * cap, hok, sizeof(int32_t) * n, cudaMemcpyHostToDevice, g->stream));
    CK(cudaEventRecord(g->staged, g->stream));
    return SBC_OK;
}

int collect_stats(sbc_forest* f, int64_t n, sbc_batch_stats* st)
{
    sbc_graph* g = f->g;
    if (!st) return SBC_OK;
    std::vector<int32_t> ok(n);
    if (n) CK(cudaMemcpyAsync(ok.data(), g->d_ins + 2 * g->ins_capacity, sizeof(int32_t) * n, cudaMemcpyDeviceToHost,
                              g->stream));
    int nwork = 0;
    CK(cudaMemcpyAsync(&nwork, f->d_nwork, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    unsigned long long c[SBC_NCOUNTERS];
    CK(cudaMemcpyAsync(c, f->d_counters, sizeof c, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemsetAsync(f->d_counters, 0, sizeof c, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    memset(st, 0, sizeof *st);
    for (int64_t i = 0; i < n; ++i) {
        if (ok[i] > 0) st->inserted++;
        else if (ok[i] == 0) st->duplicates++;
        else st->invalid++;
    }
    st->roots_active = nwork;
    st->vertices = (int64_t)c[0];
    st->edges = (int64_t)c[1];
    st->case1 = (int64_t)c[2];
    st->case2 = (int64_t)c[3];
    st->scanned = (int64_t)c[4];
    return SBC_OK;
}

// One device-input batch: the endpoints' addresses are recorded on the stream
// (k_set_src), then staging, append, classify, update and seal run from a CUDA
// graph captured once per batch size n and replayed unchanged.  Falls back to
// direct launches (and stops capturing) if the capture is refused.
int launch_batch_direct(sbc_forest* f, int n)
{
    sbc_graph* g = f->g;
    CK(sbc::launch_stage(g, n));
    CK(sbc::launch_append(g, n, false));
    CK(sbc::launch_update(f, n, false));
    CK(sbc::launch_seal(g, n));
    return SBC_OK;
}

int replay_batch(sbc_forest* f, int n, const int32_t* d_u, const int32_t* d_v)
{
    sbc_graph* g = f->g;
    CK(sbc::launch_set_src(g, d_u, d_v));
    sbc_forest::CapturedBatch* cb = nullptr;
    for (auto& p : f->captured)
        if (p.first == n) cb = &p.second;
    if (cb && cb->exec && (cb->repacks != g->repacks || cb->d_ins != g->d_ins)) {
        cudaGraphExecDestroy(cb->exec);
        cb->exec = nullptr;
    }
    if (!cb || !cb->exec) {
        if (!cb) {
            f->captured.emplace_back(n, sbc_forest::CapturedBatch());
            cb = &f->captured.back().second;
        }
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal);
        if (!e) {
            cudaError_t el = sbc::launch_stage(g, n);
            if (!el) el = sbc::launch_append(g, n, false);
            if (!el) el = sbc::launch_update(f, n, false);
            if (!el) el = sbc::launch_seal(g, n);
            e = cudaStreamEndCapture(g->stream, &graph);
            if (!e) e = el;
        }
        if (!e) e = cudaGraphInstantiate(&cb->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e) {
            cudaGetLastError();
            if (cb->exec) cudaGraphExecDestroy(cb->exec);
            cb->exec = nullptr;
            f->use_graphs = false;  // capture refused here: launch directly from now on
            return launch_batch_direct(f, n);
        }
        cb->repacks = g->repacks;
        cb->d_ins = g->d_ins;
    }
    CK(cudaGraphLaunch(cb->exec, g->stream));
    return SBC_OK;
}

int check_graph_err(sbc_graph* g)
{
    int err = 0;
    CK(cudaMemcpyAsync(&err, g->d_err, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    if (err) {
        cudaMemsetAsync(g->d_err, 0, sizeof(int), g->stream);
        return fail(SBC_ERR_STATE, "adjacency slack exhausted during an insertion batch (reserve capacity first)");
    }
    return SBC_OK;
}

void free_scratch(sbc_forest* f)
{
    f->ws.release();
    f->workers = 0;
    f->bytes = f->state_bytes;
}

void drop_captured(sbc_forest* f)
{
    for (auto& p : f->captured)
        if (p.second.exec) cudaGraphExecDestroy(p.second.exec);
    f->captured.clear();
}

void free_model(sbc_forest* f)
{
    CostModel* M = f->model;
    if (!M) return;
    dev_free(M->d_params);
    dev_free(M->d_m);
    dev_free(M->d_v);
    dev_free(M->d_grad);
    dev_free(M->d_x);
    dev_free(M->d_y);
    dev_free(M->d_n);
    dev_free(M->d_sums);
    dev_free(M->d_feat);
    dev_free(M->d_cost_log);
    dev_free(M->d_root_cost);
    dev_free(M->d_buckets);
    delete M;
    f->model = nullptr;
}

// The cost model's parameters, optimiser state and accumulators, on first use.
int ensure_model(sbc_forest* f)
{
    if (f->model) return SBC_OK;
    CostModel* M = new CostModel();
    f->model = M;
    cudaError_t e;
    if ((e = dev_alloc(&M->d_params, sbc::kModelParams)) || (e = dev_alloc(&M->d_m, sbc::kTrainParams)) ||
        (e = dev_alloc(&M->d_v, sbc::kTrainParams)) || (e = dev_alloc(&M->d_grad, sbc::kTrainParams)) ||
        (e = dev_alloc(&M->d_n, 1)) || (e = dev_alloc(&M->d_sums, 32)) || (e = dev_alloc(&M->d_root_cost, f->nk)) ||
        (e = dev_alloc(&M->d_buckets, sbc::kCostBuckets)) ||
        (e = cudaMemsetAsync(M->d_params, 0, sizeof(float) * sbc::kModelParams, f->g->stream)) ||
        (e = cudaMemsetAsync(M->d_grad, 0, sizeof(float) * sbc::kTrainParams, f->g->stream)) ||
        (e = cudaMemsetAsync(M->d_n, 0, sizeof(unsigned long long), f->g->stream))) {
        free_model(f);
        return cuda_fail(e, "cost model allocation");
    }
    return SBC_OK;
}

// Per-batch log buffers (features and costs of every (root, insertion) pair)
// for batches of up to n insertions.  Captured batch graphs hold the old
// buffers, so they are dropped when the buffers move.
int ensure_model_batch(sbc_forest* f, int64_t n)
{
    CostModel* M = f->model;
    if (!M || !M->logging || M->log_ins >= n) return SBC_OK;
    dev_free(M->d_feat);
    dev_free(M->d_cost_log);
    M->log_ins = 0;
    cudaError_t e;
    const size_t pairs = (size_t)f->nk * (size_t)n;
    if ((e = dev_alloc(&M->d_feat, pairs * sbc::kIn)) || (e = dev_alloc(&M->d_cost_log, pairs)))
        return cuda_fail(e, "cost log buffers");
    M->log_ins = n;
    drop_captured(f);
    return SBC_OK;
}

size_t scratch_per_worker(int64_t nv) { return WorkerScratch::per_worker(nv); }

// Worker count of launch shape `variant`: one per CTA the update kernel keeps
// resident (or the caller's count), at most one per root, and at most as many
// as half of `free_b` holds.
int64_t workers_for(const sbc_forest* f, int variant, size_t free_b)
{
    int per_sm = sbc::update_workers_per_sm(variant);
    if (per_sm < 1) per_sm = 1;
    int64_t w = f->workers_req > 0 ? f->workers_req : (int64_t)per_sm * f->sm_count;
    const int64_t fit = (int64_t)((free_b / 2) / scratch_per_worker(f->nv));
    w = std::min<int64_t>(w, std::max<int64_t>(fit, 1));
    w = std::min<int64_t>(w, f->nk);
    return std::max<int64_t>(w, 1);
}

// (Re)allocates the persistent workers' scratch for launch shape `variant`
// and zeroes it (every job leaves the scratch it touched zeroed again).  The
// static kernel runs over the same worker slots.  Captured batch graphs hold
// the old shape, so they are dropped.
int alloc_scratch(sbc_forest* f, int variant)
{
    sbc_graph* g = f->g;
    free_scratch(f);
    drop_captured(f);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const int64_t w = workers_for(f, variant, free_b);
    cudaError_t e = f->ws.alloc(w, f->nv, g->stream);
    if (e) {
        free_scratch(f);
        return cuda_fail(e, "worker scratch allocation");
    }
    f->variant = variant;
    f->workers = w;
    f->bytes = f->state_bytes + (int64_t)f->ws.bytes();
    return SBC_OK;
}

// A copy of the first nk rows of a forest's state (and its BC) that an
// autotuner's timing runs work on: swap() exchanges it with the forest's own
// arrays, so a launch between two swaps updates the copy only.
struct TrialState {
    int64_t nk = 0;
    int32_t* dist = nullptr;
    uint8_t* dist8 = nullptr;
    uint32_t* dist2 = nullptr;
    int64_t* sigma = nullptr;
    double* delta = nullptr;
    double* bc = nullptr;
    int32_t* hist = nullptr;
    int32_t *roster = nullptr, *roster_n = nullptr, *roster_dirty = nullptr;
    cudaError_t alloc(const sbc_forest* f, int64_t rows)
    {
        nk = rows;
        const size_t cells = (size_t)rows * (size_t)f->nv;
        cudaError_t e;
        if ((e = dev_alloc(&dist, cells)) || (e = dev_alloc(&dist8, cells)) ||
            (e = dev_alloc(&dist2, (size_t)rows * (size_t)sbc::d2_words(f->nv))) || (e = dev_alloc(&sigma, cells)) ||
            (e = dev_alloc(&delta, cells)) || (e = dev_alloc(&bc, f->nv)) ||
            (f->d_lvlhist && (e = dev_alloc(&hist, (size_t)rows * sbc::kHistLevels))) ||
            (f->d_roster && ((e = dev_alloc(&roster, (size_t)rows * sbc::kRosterLevels * sbc::kRosterCap)) ||
                             (e = dev_alloc(&roster_n, (size_t)rows * sbc::kRosterLevels)) ||
                             (e = dev_alloc(&roster_dirty, (size_t)rows * sbc::kRosterLevels)))))
            release();
        return e;
    }
    void release()
    {
        dev_free(dist);
        dev_free(dist8);
        dev_free(dist2);
        dev_free(sigma);
        dev_free(delta);
        dev_free(bc);
        dev_free(hist);
        dev_free(roster);
        dev_free(roster_n);
        dev_free(roster_dirty);
    }
    cudaError_t copy_from(const sbc_forest* f, cudaStream_t s) const
    {
        const size_t cells = (size_t)nk * (size_t)f->nv;
        const auto d2d = cudaMemcpyDeviceToDevice;
        cudaError_t e;
        if ((e = cudaMemcpyAsync(dist, f->d_dist, sizeof(int32_t) * cells, d2d, s)) ||
            (e = cudaMemcpyAsync(dist8, f->d_dist8, cells, d2d, s)) ||
            (e = cudaMemcpyAsync(dist2, f->d_dist2, sizeof(uint32_t) * (size_t)nk * (size_t)sbc::d2_words(f->nv), d2d,
                                 s)) ||
            (e = cudaMemcpyAsync(sigma, f->d_sigma, sizeof(int64_t) * cells, d2d, s)) ||
            (e = cudaMemcpyAsync(delta, f->d_delta, sizeof(double) * cells, d2d, s)) ||
            (e = cudaMemcpyAsync(bc, f->d_bc, sizeof(double) * f->nv, d2d, s)) ||
            (hist && (e = cudaMemcpyAsync(hist, f->d_lvlhist, sizeof(int32_t) * (size_t)nk * sbc::kHistLevels, d2d, s))) ||
            (roster && ((e = cudaMemcpyAsync(roster, f->d_roster,
                                             sizeof(int32_t) * (size_t)nk * sbc::kRosterLevels * sbc::kRosterCap, d2d, s)) ||
                        (e = cudaMemcpyAsync(roster_n, f->d_roster_n, sizeof(int32_t) * (size_t)nk * sbc::kRosterLevels,
                                             d2d, s)) ||
                        (e = cudaMemcpyAsync(roster_dirty, f->d_roster_dirty,
                                             sizeof(int32_t) * (size_t)nk * sbc::kRosterLevels, d2d, s)))))
            return e;
        return cudaSuccess;
    }
    void swap(sbc_forest* f)
    {
        std::swap(f->d_dist, dist);
        std::swap(f->d_dist8, dist8);
        std::swap(f->d_dist2, dist2);
        std::swap(f->d_sigma, sigma);
        std::swap(f->d_delta, delta);
        std::swap(f->d_bc, bc);
        if (hist) std::swap(f->d_lvlhist, hist);
        if (roster) {
            std::swap(f->d_roster, roster);
            std::swap(f->d_roster_n, roster_n);
            std::swap(f->d_roster_dirty, roster_dirty);
        }
        std::swap(f->nk, nk);
    }
};

// ---- groups ----

void group_free_scratch(sbc_group* G) { G->ws.release(); }

// Worker scratch of the group for shape `variant`: one worker per resident
// CTA, at most one per root of all members, within half the free memory.
int group_alloc_scratch(sbc_group* G, int variant)
{
    G->ws.release();
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const int per_sm = std::max(1, sbc::group_workers_per_sm(variant));
    int64_t w = (int64_t)per_sm * G->sm_count;
    w = std::min<int64_t>(w, std::max<int64_t>((int64_t)((free_b / 2) / WorkerScratch::per_worker(G->nv_max)), 1));
    w = std::max<int64_t>(std::min<int64_t>(w, G->total_roots), 1);
    cudaError_t e = G->ws.alloc(w, G->nv_max, G->stream);
    if (e) return cuda_fail(e, "group worker scratch allocation");
    G->variant = variant;
    return SBC_OK;
}

// Work queued on the members' graph streams precedes what is queued next on
// the group's stream, and vice versa.
int group_after_members(sbc_group* G)
{
    for (sbc_forest* f : G->members) {
        CK(cudaEventRecord(G->ev, f->g->stream));
        CK(cudaStreamWaitEvent(G->stream, G->ev, 0));
    }
    return SBC_OK;
}

int members_after_group(sbc_group* G)
{
    CK(cudaEventRecord(G->ev, G->stream));
    for (sbc_forest* f : G->members) CK(cudaStreamWaitEvent(f->g->stream, G->ev, 0));
    return SBC_OK;
}

// Validates the per-member counts (caller order), plans slack and stages each
// member's insertions in its graph; counts_slot[s] receives slot s's count.
int group_stage(sbc_group* G, const int64_t* counts, const int64_t* u, const int64_t* v, std::vector<int>& counts_slot)
{
    const int ns = (int)G->members.size();
    std::vector<int64_t> off(ns + 1, 0);
    for (int i = 0; i < ns; ++i) {
        if (counts[i] < 0 || counts[i] >= INT32_MAX) return fail(SBC_ERR_ARG, "group batch: bad count for member %d", i);
        off[i + 1] = off[i] + counts[i];
    }
    if (off[ns] > 0 && (!u || !v)) return fail(SBC_ERR_ARG, "group batch: null endpoints");
    counts_slot.assign(ns, 0);
    for (int s = 0; s < ns; ++s) {
        const int m = G->order[s];
        const int64_t n = counts[m];
        counts_slot[s] = (int)n;
        if (n == 0) continue;
        sbc_graph* g = G->members[s]->g;
        int rc = plan_capacity(g, n, u + off[m], v + off[m], false);
        if (rc) return rc;
        if ((rc = stage_host(g, n, u + off[m], v + off[m], false))) return rc;
    }
    return SBC_OK;
}

int group_check(sbc_group* G)
{
    if (!G) return fail(SBC_ERR_ARG, "group: null");
    for (sbc_forest* f : G->members)
        if (!f->g) return fail(SBC_ERR_STATE, "group: a member's graph was destroyed");
    return use_device(G->device);
}

template <class T>
int get_rows(sbc_forest* f, const T* base, int64_t r0, int64_t nr, T* out)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "state read: the forest's graph was destroyed");
    if (!f || !out || r0 < 0 || nr < 0 || r0 + nr > f->nk) return fail(SBC_ERR_ARG, "state read: bad row range");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaMemcpyAsync(out, base + (size_t)r0 * f->nv, sizeof(T) * (size_t)nr * f->nv, cudaMemcpyDeviceToHost,
                       f->g->stream));
    CK(cudaStreamSynchronize(f->g->stream));
    return SBC_OK;
}

}  // namespace

namespace sbc {

int report_error(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return fail(code, "%s", buf);
}

}  // namespace sbc

extern "C" {

const char* sbc_last_error(void) { return t_err.c_str(); }

int sbc_set_device(int device)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(SBC_ERR_NOGPU, "no CUDA device");
    if (device < 0 || device >= n) return fail(SBC_ERR_ARG, "device %d out of range", device);
    t_device = device;
    return use_device(device);
}

// ------------------------------------------------------------------ graph

int sbc_graph_create(sbc_graph** out, int64_t nv, const int64_t* off, const int64_t* adj)
{
    if (!out || nv < 0 || nv >= INT32_MAX || !off || (off[nv] > 0 && !adj)) return fail(SBC_ERR_ARG, "sbc_graph_create: bad arguments");
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(SBC_ERR_NOGPU, "no CUDA device");
    const int dev = current_device();
    if (use_device(dev)) return SBC_ERR_CUDA;
    for (int64_t v = 0; v < nv; ++v)
        if (off[v + 1] < off[v]) return fail(SBC_ERR_ARG, "sbc_graph_create: offsets not monotone at %lld", (long long)v);
    for (int64_t e = 0; e < off[nv]; ++e)
        if (adj[e] < 0 || adj[e] >= nv) return fail(SBC_ERR_ARG, "sbc_graph_create: neighbour id out of range at %lld", (long long)e);

    sbc_graph* g = new sbc_graph();
    g->device = dev;
    g->nv = nv;
    g->h_row.resize(nv + 1);
    g->h_cap.resize(nv);
    g->h_deg_ub.resize(nv);
    std::vector<int32_t> deg(nv);
    int64_t total = 0;
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t d = off[v + 1] - off[v];
        if (d >= INT32_MAX - 8) {
            delete g;
            return fail(SBC_ERR_ARG, "degree too large");
        }
        deg[v] = (int32_t)d;
        g->h_row[v] = total;
        g->h_cap[v] = slack_cap(d);
        g->h_deg_ub[v] = d;
        total += g->h_cap[v];
    }
    g->h_row[nv] = total;
    g->total_cap = total;

    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&g->staged, cudaEventDisableTiming)) || (e = dev_alloc(&g->d_row, nv + 1)) ||
        (e = dev_alloc(&g->d_deg, nv)) || (e = dev_alloc(&g->d_deg0, nv)) || (e = dev_alloc(&g->d_cap, nv)) ||
        (e = dev_alloc(&g->d_nsort, nv)) ||
        (e = dev_alloc(&g->d_col, total)) || (e = dev_alloc(&g->d_seq, total)) || (e = dev_alloc(&g->d_err, 2)) ||
        (e = dev_alloc(&g->d_src, 2))) {
        sbc_graph_destroy(g);
        return cuda_fail(e, "sbc_graph_create allocation");
    }
    if ((e = cudaMemcpy(g->d_row, g->h_row.data(), sizeof(int64_t) * (nv + 1), cudaMemcpyHostToDevice)) ||
        (nv && (e = cudaMemcpy(g->d_deg, deg.data(), sizeof(int32_t) * nv, cudaMemcpyHostToDevice))) ||
        (nv && (e = cudaMemcpy(g->d_deg0, deg.data(), sizeof(int32_t) * nv, cudaMemcpyHostToDevice))) ||
        (nv && (e = cudaMemcpy(g->d_nsort, deg.data(), sizeof(int32_t) * nv, cudaMemcpyHostToDevice))) ||
        (nv && (e = cudaMemcpy(g->d_cap, g->h_cap.data(), sizeof(int32_t) * nv, cudaMemcpyHostToDevice))) ||
        (e = cudaMemset(g->d_col, 0, sizeof(int32_t) * std::max<int64_t>(total, 1))) ||
        (e = cudaMemset(g->d_seq, 0, sizeof(int32_t) * std::max<int64_t>(total, 1))) ||
        (e = cudaMemset(g->d_err, 0, 2 * sizeof(int)))) {
        sbc_graph_destroy(g);
        return cuda_fail(e, "sbc_graph_create upload");
    }
    // Each vertex's initial neighbours are stored sorted, so adjacency can be
    // tested by binary search (insertions later append an unsorted tail); the
    // scatter into the slack layout and the sort run on the device.
    {
        int sm_count = 0;
        cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
        if ((e = sbc::build_adjacency(nv, off, adj, g->d_row, g->d_deg, deg, g->d_col, std::max(sm_count, 1),
                                      g->stream))) {
            sbc_graph_destroy(g);
            return cuda_fail(e, "sbc_graph_create adjacency build");
        }
    }
    int rc = ensure_staging(g, 64);
    if (rc) {
        sbc_graph_destroy(g);
        return rc;
    }
    *out = g;
    return SBC_OK;
}

int sbc_graph_destroy(sbc_graph* g)
{
    if (!g) return SBC_OK;
    use_device(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    for (sbc_forest* f : g->forests) f->g = nullptr;  // forests outliving their graph are detached
    dev_free(g->d_row);
    dev_free(g->d_deg);
    dev_free(g->d_deg0);
    dev_free(g->d_nsort);
    dev_free(g->d_cap);
    dev_free(g->d_col);
    dev_free(g->d_seq);
    dev_free(g->d_err);
    dev_free(g->d_src);
    dev_free(g->d_ins);
    if (g->h_ins) cudaFreeHost(g->h_ins);
    if (g->staged) cudaEventDestroy(g->staged);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return SBC_OK;
}

int sbc_graph_num_vertices(const sbc_graph* g, int64_t* nv)
{
    if (!g || !nv) return fail(SBC_ERR_ARG, "sbc_graph_num_vertices: null");
    *nv = g->nv;
    return SBC_OK;
}

int sbc_graph_degree(sbc_graph* g, int64_t v, int64_t* deg)
{
    if (!g || !deg || v < 0 || v >= g->nv) return fail(SBC_ERR_ARG, "sbc_graph_degree: bad arguments");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    int32_t d = 0;
    CK(cudaMemcpyAsync(&d, g->d_deg + v, sizeof d, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    *deg = d;
    return SBC_OK;
}

int sbc_graph_insert_directed(sbc_graph* g, int64_t from, int64_t to, int* result)
{
    if (!g) return fail(SBC_ERR_ARG, "sbc_graph_insert_directed: null graph");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    int rc = plan_capacity(g, 1, &from, &to, true);
    if (rc) return rc;
    if ((rc = stage_host(g, 1, &from, &to, false))) return rc;
    CK(sbc::launch_append(g, 1, true));
    CK(sbc::launch_seal(g, 1));
    int32_t code = 0;
    CK(cudaMemcpyAsync(&code, g->d_ins + 2 * g->ins_capacity, sizeof code, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    if (code == -2) return check_graph_err(g);
    if (result) *result = code < 0 ? -1 : code;
    return SBC_OK;
}

int sbc_graph_reserve(sbc_graph* g, int64_t n, const int64_t* u, const int64_t* v)
{
    if (!g || n < 0 || (n > 0 && (!u || !v))) return fail(SBC_ERR_ARG, "sbc_graph_reserve: bad arguments");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    return plan_capacity(g, n, u, v, false);
}

int sbc_graph_repacks(const sbc_graph* g, int64_t* count)
{
    if (!g || !count) return fail(SBC_ERR_ARG, "sbc_graph_repacks: null");
    *count = g->repacks;
    return SBC_OK;
}

int sbc_graph_to_csr(sbc_graph* g, int64_t* off, int64_t* adj)
{
    if (!g || !off) return fail(SBC_ERR_ARG, "sbc_graph_to_csr: null");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    CK(cudaStreamSynchronize(g->stream));
    std::vector<int32_t> deg(g->nv);
    if (g->nv) CK(cudaMemcpy(deg.data(), g->d_deg, sizeof(int32_t) * g->nv, cudaMemcpyDeviceToHost));
    off[0] = 0;
    for (int64_t v = 0; v < g->nv; ++v) off[v + 1] = off[v] + deg[v];
    if (!adj) return SBC_OK;
    std::vector<int32_t> col(g->total_cap > 0 ? g->total_cap : 1);
    CK(cudaMemcpy(col.data(), g->d_col, sizeof(int32_t) * col.size(), cudaMemcpyDeviceToHost));
    for (int64_t v = 0; v < g->nv; ++v)
        for (int32_t s = 0; s < deg[v]; ++s) adj[off[v] + s] = col[g->h_row[v] + s];
    return SBC_OK;
}

// ------------------------------------------------------------------ forest

int sbc_update_variant_count(int* count)
{
    if (!count) return fail(SBC_ERR_ARG, "sbc_update_variant_count: null");
    *count = sbc::update_variant_count();
    return SBC_OK;
}

int sbc_update_variant_info(int v, int* threads_per_cta, int* min_ctas_per_sm, int* ctas_per_sm)
{
    if (v < 0 || v >= sbc::update_variant_count()) return fail(SBC_ERR_ARG, "update variant %d out of range", v);
    if (threads_per_cta) *threads_per_cta = sbc::update_variant_threads(v);
    if (min_ctas_per_sm) *min_ctas_per_sm = 0;
    if (ctas_per_sm) *ctas_per_sm = sbc::update_workers_per_sm(v);
    return SBC_OK;
}

int sbc_forest_create(sbc_forest** out, sbc_graph* g, int64_t nk, const int64_t* roots, int64_t workers)
{
    return sbc_forest_create_ex(out, g, nk, roots, workers, -1);
}

int sbc_forest_create_ex(sbc_forest** out, sbc_graph* g, int64_t nk, const int64_t* roots, int64_t workers,
                         int variant)
{
    if (!out || !g || nk <= 0 || !roots) return fail(SBC_ERR_ARG, "sbc_forest_create: bad arguments");
    *out = nullptr;
    if (variant < 0) {
        const char* env = getenv("SBC_UPDATE_VARIANT");
        variant = env ? atoi(env) : sbc::update_default_variant();
    }
    if (variant < 0 || variant >= sbc::update_variant_count())
        return fail(SBC_ERR_ARG, "update variant %d out of range", variant);
    if (nk > g->nv) return fail(SBC_ERR_ARG, "more roots (%lld) than vertices (%lld)", (long long)nk, (long long)g->nv);
    if (nk >= INT32_MAX) return fail(SBC_ERR_ARG, "too many roots");
    {
        std::vector<char> seen(g->nv, 0);
        for (int64_t r = 0; r < nk; ++r) {
            if (roots[r] < 0 || roots[r] >= g->nv) return fail(SBC_ERR_ARG, "root %lld out of range", (long long)roots[r]);
            if (seen[roots[r]]) return fail(SBC_ERR_ARG, "root %lld repeated", (long long)roots[r]);
            seen[roots[r]] = 1;
        }
    }
    if (use_device(g->device)) return SBC_ERR_CUDA;
    sbc_forest* f = new sbc_forest();
    f->g = g;
    f->device = g->device;
    f->nv = g->nv;
    f->nk = nk;
    f->variant = variant;
    f->h_roots.assign(roots, roots + nk);
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, g->device));
    f->sm_count = prop.multiProcessorCount;
    const size_t cells = (size_t)nk * (size_t)f->nv;
    cudaError_t e;
    if ((e = dev_alloc(&f->d_roots, nk)) || (e = dev_alloc(&f->d_dist, cells)) || (e = dev_alloc(&f->d_dist8, cells)) ||
        (e = dev_alloc(&f->d_dist2, (size_t)nk * (size_t)sbc::d2_words(f->nv))) || (e = dev_alloc(&f->d_sigma, cells)) ||
        (e = dev_alloc(&f->d_delta, cells)) || (e = dev_alloc(&f->d_bc, f->nv)) || (e = dev_alloc(&f->d_worklist, nk)) ||
        (e = dev_alloc(&f->d_nwork, 2)) || (e = dev_alloc(&f->d_counters, SBC_NCOUNTERS)) ||
        (e = dev_alloc(&f->d_mov, nk)) || (e = dev_alloc(&f->d_nmov, 2)) || (e = dev_alloc(&f->d_dirty, nk)) ||
        (e = dev_alloc(&f->d_dlist, nk)) || (e = dev_alloc(&f->d_dcnt, 1)) ||
        (e = dev_alloc(&f->d_lvlhist, (size_t)nk * sbc::kHistLevels))) {
        sbc_forest_destroy(f);
        return cuda_fail(e, "sbc_forest_create state allocation");
    }
    f->d_counter = f->d_nwork + 1;
    // rosters (16 KB per root) unless they would take more than 1 GB
    const size_t roster_cells = (size_t)nk * sbc::kRosterLevels * sbc::kRosterCap;
    if (roster_cells * 4 <= ((size_t)1 << 30) &&
        ((e = dev_alloc(&f->d_roster, roster_cells)) ||
         (e = dev_alloc(&f->d_roster_n, (size_t)nk * sbc::kRosterLevels)) ||
         (e = dev_alloc(&f->d_roster_dirty, (size_t)nk * sbc::kRosterLevels)))) {
        sbc_forest_destroy(f);
        return cuda_fail(e, "sbc_forest_create roster allocation");
    }
    // level-2 parent masks (4 B per root per vertex) where they take at most a
    // quarter of the free memory
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && cells * 4 <= free_b / 4) {
        if ((e = dev_alloc(&f->d_l2mask, cells)) || (e = dev_alloc(&f->d_l1cand, (size_t)nk * sbc::kL1Max)) ||
            (e = dev_alloc(&f->d_l1n, nk)) || (e = dev_alloc(&f->d_l2flag, nk)) || (e = dev_alloc(&f->d_l2list, nk)) ||
            (e = dev_alloc(&f->d_l2cnt, 1))) {
            sbc_forest_destroy(f);
            return cuda_fail(e, "sbc_forest_create mask allocation");
        }
        CK(cudaMemsetAsync(f->d_l1n, 0xff, sizeof(int32_t) * nk, g->stream));  // -1: no masks until built
        CK(cudaMemsetAsync(f->d_l2flag, 0, sizeof(int32_t) * nk, g->stream));
        CK(cudaMemsetAsync(f->d_l2cnt, 0, sizeof(int32_t), g->stream));
    }
    f->state_bytes = (int64_t)(cells * 21 + (size_t)nk * sbc::d2_words(f->nv) * 4 + f->nv * 8 +
                               (f->d_roster ? roster_cells * 4 : 0) + (f->d_l2mask ? cells * 4 : 0));
    f->workers_req = workers;
    int rc = alloc_scratch(f, variant);
    if (rc) {
        sbc_forest_destroy(f);
        return rc;
    }
    CK(cudaMemsetAsync(f->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, g->stream));
    CK(cudaMemsetAsync(f->d_dirty, 0, sizeof(int) * nk, g->stream));
    CK(cudaMemsetAsync(f->d_dcnt, 0, sizeof(int), g->stream));
    CK(cudaMemcpyAsync(f->d_roots, roots, sizeof(int64_t) * nk, cudaMemcpyHostToDevice, g->stream));
    CK(f->prof_init());
    CK(cudaEventCreate(&f->t0));
    CK(cudaEventCreate(&f->t1));
    CK(cudaStreamSynchronize(g->stream));
    g->forests.push_back(f);
    *out = f;
    return SBC_OK;
}

int sbc_forest_destroy(sbc_forest* f)
{
    if (!f) return SBC_OK;
    if (f->groups > 0) return fail(SBC_ERR_STATE, "sbc_forest_destroy: the forest is a member of a live group");
    use_device(f->device);
    if (f->g) {
        cudaStreamSynchronize(f->g->stream);
        auto& fs = f->g->forests;
        fs.erase(std::remove(fs.begin(), fs.end(), f), fs.end());
    }
    dev_free(f->d_roots);
    dev_free(f->d_dist);
    dev_free(f->d_dist8);
    dev_free(f->d_dist2);
    dev_free(f->d_l2mask);
    dev_free(f->d_l1cand);
    dev_free(f->d_l1n);
    dev_free(f->d_l2flag);
    dev_free(f->d_l2list);
    dev_free(f->d_l2cnt);
    dev_free(f->d_sigma);
    dev_free(f->d_delta);
    dev_free(f->d_bc);
    dev_free(f->d_worklist);
    dev_free(f->d_nwork);
    dev_free(f->d_counters);
    dev_free(f->d_lvlhist);
    dev_free(f->d_mov);
    dev_free(f->d_dirty);
    dev_free(f->d_dlist);
    dev_free(f->d_dcnt);
    dev_free(f->d_wide);
    dev_free(f->d_nmov);
    dev_free(f->d_roster);
    dev_free(f->d_roster_n);
    dev_free(f->d_roster_dirty);
    free_model(f);
    free_scratch(f);
    f->prof_release();
    drop_captured(f);
    if (f->t0) cudaEventDestroy(f->t0);
    if (f->t1) cudaEventDestroy(f->t1);
    delete f;
    return SBC_OK;
}

int sbc_forest_info(const sbc_forest* f, int64_t* nv, int64_t* nk, int64_t* workers, int64_t* bytes)
{
    if (!f) return fail(SBC_ERR_ARG, "sbc_forest_info: null");
    if (nv) *nv = f->nv;
    if (nk) *nk = f->nk;
    if (workers) *workers = f->workers;
    if (bytes) *bytes = f->bytes;
    return SBC_OK;
}

int sbc_static_init(sbc_forest* f)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_static_init: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_static_init: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(sbc::launch_static(f));
    CK(sbc::launch_dist2_rows(f, nullptr, nullptr));
    CK(sbc::launch_l2mask_build_all(f));
    CK(sbc::launch_level_hist(f));
    CK(sbc::launch_roster_build(f));
    f->initialized = true;
    return SBC_OK;
}

int sbc_insert_batch(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v, sbc_batch_stats* stats)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_insert_batch: the forest's graph was destroyed");
    if (!f || n < 0 || (n > 0 && (!u || !v))) return fail(SBC_ERR_ARG, "sbc_insert_batch: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_insert_batch before sbc_static_init");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (n == 0) {
        if (stats) memset(stats, 0, sizeof *stats);
        return SBC_OK;
    }
    int rc = plan_capacity(g, n, u, v, false);
    if (rc) return rc;
    if ((rc = stage_host(g, n, u, v, false))) return rc;
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    // per-call statistics cover this call only
    if (stats) CK(cudaMemsetAsync(f->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, g->stream));
    f->prof_begin(sbc::PROF_BATCH);
    f->prof_begin(sbc::PROF_APPEND);
    CK(sbc::launch_append(g, (int)n, false));
    f->prof_end(sbc::PROF_APPEND);
    CK(sbc::launch_update(f, (int)n, false));
    CK(sbc::launch_seal(g, (int)n));
    f->prof_end(sbc::PROF_BATCH);
    if ((rc = collect_stats(f, n, stats))) return rc;
    return check_graph_err(g);
}

int sbc_insert_batch_async(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_insert_batch_async: the forest's graph was destroyed");
    if (!f || n < 0 || (n > 0 && (!u || !v))) return fail(SBC_ERR_ARG, "sbc_insert_batch_async: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_insert_batch_async before sbc_static_init");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    if (n == 0) return SBC_OK;
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    int rc = plan_capacity(g, n, u, v, false);
    if (rc) return rc;
    if ((rc = stage_host(g, n, u, v, false))) return rc;
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    CK(sbc::launch_append(g, (int)n, false));
    CK(sbc::launch_update(f, (int)n, false));
    CK(sbc::launch_seal(g, (int)n));
    return SBC_OK;
}

int sbc_insert_batch_device(sbc_forest* f, int64_t n, const int32_t* d_u, const int32_t* d_v)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_insert_batch_device: the forest's graph was destroyed");
    if (!f || n < 0 || (n > 0 && (!d_u || !d_v))) return fail(SBC_ERR_ARG, "sbc_insert_batch_device: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_insert_batch_device before sbc_static_init");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    if (n == 0) return SBC_OK;
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    int rc = ensure_staging(g, n);
    if (rc) return rc;
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    if (f->use_graphs && !f->prof) return replay_batch(f, (int)n, d_u, d_v);
    f->prof_begin(sbc::PROF_BATCH);
    CK(sbc::launch_set_src(g, d_u, d_v));
    CK(sbc::launch_stage(g, (int)n));
    f->prof_begin(sbc::PROF_APPEND);
    CK(sbc::launch_append(g, (int)n, false));
    f->prof_end(sbc::PROF_APPEND);
    CK(sbc::launch_update(f, (int)n, false));
    CK(sbc::launch_seal(g, (int)n));
    f->prof_end(sbc::PROF_BATCH);
    return SBC_OK;
}

int sbc_set_graph_capture(sbc_forest* f, int on)
{
    if (!f) return fail(SBC_ERR_ARG, "sbc_set_graph_capture: null");
    f->use_graphs = on != 0;
    return SBC_OK;
}

int sbc_forest_roots(const sbc_forest* f, int64_t* roots)
{
    if (!f || !roots) return fail(SBC_ERR_ARG, "sbc_forest_roots: null");
    std::copy(f->h_roots.begin(), f->h_roots.end(), roots);
    return SBC_OK;
}

int sbc_forest_set_variant(sbc_forest* f, int variant)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_forest_set_variant: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_forest_set_variant: null");
    if (variant < 0 || variant >= sbc::update_variant_count())
        return fail(SBC_ERR_ARG, "update variant %d out of range", variant);
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    if (variant == f->variant && f->workers > 0) return SBC_OK;
    CK(cudaStreamSynchronize(f->g->stream));
    int rc = alloc_scratch(f, variant);
    if (rc) return rc;
    CK(cudaStreamSynchronize(f->g->stream));
    return SBC_OK;
}

int sbc_forest_set_delete_mode(sbc_forest* f, int mode)
{
    if (!f || mode < SBC_DELETE_AUTO || mode > SBC_DELETE_RECOMPUTE)
        return fail(SBC_ERR_ARG, "sbc_forest_set_delete_mode: bad arguments");
    f->delete_mode = mode;
    return SBC_OK;
}

int sbc_forest_variant(const sbc_forest* f, int* variant)
{
    if (!f || !variant) return fail(SBC_ERR_ARG, "sbc_forest_variant: null");
    *variant = f->variant;
    return SBC_OK;
}

int sbc_forest_autotune(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v, int reps, int* chosen,
                        double* ms, int ms_len)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_forest_autotune: the forest's graph was destroyed");
    if (!f || n <= 0 || !u || !v || reps < 0 || ms_len < 0 || (ms_len > 0 && !ms))
        return fail(SBC_ERR_ARG, "sbc_forest_autotune: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_forest_autotune before sbc_static_init");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (reps == 0) reps = 2;
    const int nvar = sbc::update_variant_count();
    for (int i = 0; i < ms_len; ++i) ms[i] = -1.0;
    int rc = plan_capacity(g, n, u, v, false);
    if (rc) return rc;
    if ((rc = stage_host(g, n, u, v, false))) return rc;
    CK(sbc::launch_append(g, (int)n, false));
    CK(cudaStreamSynchronize(g->stream));

    // Trial copy of the state: all roots if it fits in half the free memory,
    // else a prefix of the (uniformly drawn) roots.
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const int64_t nk_t = std::min<int64_t>(f->nk, (int64_t)((free_b / 2) / ((size_t)f->nv * 21)));
    if (nk_t < 1) return fail(SBC_ERR_CUDA, "sbc_forest_autotune: no memory for a trial copy of one root");
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    const bool logging = f->model && f->model->logging;
    if (logging) f->model->logging = false;  // timing runs log nothing
    TrialState T;
    unsigned long long saved_counters[SBC_NCOUNTERS];
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool prof = f->prof;
    const int old_variant = f->variant;
    int best = -1;
    double best_ms = 0.0;
    cudaError_t e;
    auto cleanup = [&]() {
        T.release();
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        f->prof = prof;
        if (logging) f->model->logging = true;
    };
    if ((e = T.alloc(f, nk_t)) || (e = cudaEventCreate(&e0)) || (e = cudaEventCreate(&e1)) ||
        (e = cudaMemcpyAsync(saved_counters, f->d_counters, sizeof saved_counters, cudaMemcpyDeviceToHost, g->stream)) ||
        (e = cudaStreamSynchronize(g->stream))) {
        cleanup();
        return cuda_fail(e, "sbc_forest_autotune setup");
    }
    f->prof = false;
    for (int c = 0; c < nvar; ++c) {
        CK(cudaMemGetInfo(&free_b, &total_b));
        // a shape runs only with its full worker count, so that its time is its own
        const int per_sm = std::max(1, sbc::update_workers_per_sm(c));
        const int64_t want = std::min<int64_t>(f->workers_req > 0 ? f->workers_req : (int64_t)per_sm * f->sm_count, f->nk);
        const size_t have = free_b + f->ws.bytes();
        if ((size_t)want * scratch_per_worker(f->nv) > have / 2) continue;
        if ((rc = alloc_scratch(f, c))) {
            cleanup();
            return rc;
        }
        double c_ms = -1.0;
        for (int rep = 0; rep < reps; ++rep) {
            if ((e = T.copy_from(f, g->stream))) {
                cleanup();
                return cuda_fail(e, "sbc_forest_autotune trial copy");
            }
            T.swap(f);
            e = cudaEventRecord(e0, g->stream);
            if (!e) e = sbc::launch_update(f, (int)n, false);
            if (!e) e = cudaEventRecord(e1, g->stream);
            T.swap(f);
            if (!e) e = cudaEventSynchronize(e1);
            float t = 0.f;
            if (!e) e = cudaEventElapsedTime(&t, e0, e1);
            if (e) {
                cleanup();
                return cuda_fail(e, "sbc_forest_autotune trial");
            }
            if (c_ms < 0.0 || t < c_ms) c_ms = t;
        }
        if (c < ms_len) ms[c] = c_ms;
        if (best < 0 || c_ms < best_ms) {
            best = c;
            best_ms = c_ms;
        }
    }
    cleanup();
    if (best < 0) best = old_variant;
    if ((rc = alloc_scratch(f, best))) return rc;
    CK(cudaMemcpyAsync(f->d_counters, saved_counters, sizeof saved_counters, cudaMemcpyHostToDevice, g->stream));
    CK(sbc::launch_update(f, (int)n, false));
    CK(sbc::launch_seal(g, (int)n));
    if (chosen) *chosen = best;
    return check_graph_err(g);
}

// ------------------------------------------------------------------ deletions

int sbc_graph_neighbors(sbc_graph* g, int64_t v, int64_t* out, int64_t cap, int64_t* n)
{
    if (!g || !n || v < 0 || v >= g->nv || cap < 0 || (cap > 0 && !out))
        return fail(SBC_ERR_ARG, "sbc_graph_neighbors: bad arguments");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    int32_t d = 0;
    CK(cudaMemcpyAsync(&d, g->d_deg + v, sizeof d, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    *n = d;
    if (cap == 0 || d == 0) return SBC_OK;
    const int64_t k = std::min<int64_t>(cap, d);
    std::vector<int32_t> buf((size_t)k);
    CK(cudaMemcpy(buf.data(), g->d_col + g->h_row[v], sizeof(int32_t) * k, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < k; ++i) out[i] = buf[i];
    return SBC_OK;
}

int sbc_graph_remove_directed(sbc_graph* g, int64_t from, int64_t to, int* result)
{
    if (!g || !result) return fail(SBC_ERR_ARG, "sbc_graph_remove_directed: bad arguments");
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (from < 0 || to < 0 || from >= g->nv || to >= g->nv || from == to) {
        *result = -1;
        return SBC_OK;
    }
    CK(sbc::launch_remove(g, (int)from, (int)to, true, g->d_err + 1));
    CK(cudaMemcpyAsync(result, g->d_err + 1, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    return SBC_OK;
}

namespace {
// Deletion statistics of one call from the per-deletion removal codes
// (staged at d_codes) and the forest's counters.
int deletion_stats(sbc_forest* f, int64_t n, const int32_t* d_codes, sbc_batch_stats* st)
{
    sbc_graph* g = f->g;
    std::vector<int32_t> codes(n);
    unsigned long long c[SBC_NCOUNTERS];
    CK(cudaMemcpyAsync(codes.data(), d_codes, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemcpyAsync(c, f->d_counters, sizeof c, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaMemsetAsync(f->d_counters, 0, sizeof c, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    memset(st, 0, sizeof *st);
    for (int32_t k : codes) {
        if (k > 0) st->inserted++;
        else if (k == 0) st->duplicates++;
        else st->invalid++;
    }
    st->vertices = (int64_t)c[0];
    st->edges = (int64_t)c[1];
    st->case1 = (int64_t)c[2];
    st->case2 = (int64_t)c[3];
    st->scanned = (int64_t)c[4];
    return SBC_OK;
}
}  // namespace

int sbc_delete_batch(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v, sbc_batch_stats* stats)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_delete_batch: the forest's graph was destroyed");
    if (!f || n < 0 || (n > 0 && (!u || !v))) return fail(SBC_ERR_ARG, "sbc_delete_batch: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_delete_batch before sbc_static_init");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (n == 0) {
        if (stats) memset(stats, 0, sizeof *stats);
        return SBC_OK;
    }
    int rc = stage_host(g, n, u, v, false);
    if (rc) return rc;
    const int32_t* codes = g->d_ins + 2 * g->ins_capacity;
    if (stats) CK(cudaMemsetAsync(f->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, g->stream));
    // the whole batch in one update launch: removals marked in order, every
    // root through the deletions in order (each job seeing the graph as it
    // stands after its deletion), the marked slots compacted, and the roots
    // left to a recompute recomputed once, on the final graph
    CK(sbc::launch_mark_removed(g, (int)n));
    CK(sbc::launch_delete_batch(f, (int)n));
    CK(sbc::launch_compact_removed(g, (int)n));
    CK(sbc::launch_delete_finish(f));
    if (stats) return deletion_stats(f, n, codes, stats);
    CK(cudaStreamSynchronize(g->stream));
    return SBC_OK;
}

int sbc_update_deleted(sbc_forest* f, int64_t u, int64_t v, sbc_batch_stats* stats)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_update_deleted: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_update_deleted: null");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_update_deleted before sbc_static_init");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (u < 0 || v < 0 || u >= g->nv || v >= g->nv || u == v) return fail(SBC_ERR_ARG, "sbc_update_deleted: bad edge");
    static const int kRemoved = 1;
    CK(cudaMemcpyAsync(g->d_err + 1, &kRemoved, sizeof(int), cudaMemcpyHostToDevice, g->stream));
    if (stats) CK(cudaMemsetAsync(f->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, g->stream));
    CK(sbc::launch_delete(f, (int)u, (int)v, g->d_err + 1));
    if (stats) return deletion_stats(f, 1, g->d_err + 1, stats);
    CK(cudaStreamSynchronize(g->stream));
    return SBC_OK;
}

// ------------------------------------------------------------------ cost model

int sbc_cost_model_size(int* n_params, int* n_features)
{
    if (n_params) *n_params = sbc::kModelParams;
    if (n_features) *n_features = sbc::kIn;
    return SBC_OK;
}

int sbc_cost_log_start(sbc_forest* f, int64_t capacity)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_cost_log_start: the forest's graph was destroyed");
    if (!f || capacity <= 0 || capacity >= ((int64_t)1 << 31))
        return fail(SBC_ERR_ARG, "sbc_cost_log_start: bad arguments");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    int rc = ensure_model(f);
    if (rc) return rc;
    CostModel* M = f->model;
    CK(cudaStreamSynchronize(f->g->stream));
    if (capacity != M->capacity) {
        dev_free(M->d_x);
        dev_free(M->d_y);
        M->capacity = 0;
        cudaError_t e;
        if ((e = dev_alloc(&M->d_x, (size_t)capacity * sbc::kIn)) || (e = dev_alloc(&M->d_y, (size_t)capacity)))
            return cuda_fail(e, "cost log allocation");
        M->capacity = capacity;
        CK(cudaMemset(M->d_n, 0, sizeof(unsigned long long)));
    }
    M->logging = true;
    drop_captured(f);
    return ensure_model_batch(f, f->g->ins_capacity);
}

int sbc_cost_log_stop(sbc_forest* f, int64_t* samples)
{
    if (!f || !f->g) return fail(SBC_ERR_ARG, "sbc_cost_log_stop: null forest or graph");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaStreamSynchronize(f->g->stream));
    if (f->model) {
        f->model->logging = false;
        drop_captured(f);
    }
    if (samples) {
        unsigned long long n = 0;
        if (f->model) CK(cudaMemcpy(&n, f->model->d_n, sizeof n, cudaMemcpyDeviceToHost));
        *samples = f->model ? std::min<int64_t>((int64_t)n, f->model->capacity) : 0;
    }
    return SBC_OK;
}

int sbc_cost_log_read(sbc_forest* f, int64_t first, int64_t count, float* x, float* y)
{
    if (!f || !f->g || !f->model || first < 0 || count < 0 || first + count > f->model->capacity)
        return fail(SBC_ERR_ARG, "sbc_cost_log_read: bad arguments");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaStreamSynchronize(f->g->stream));
    if (x) CK(cudaMemcpy(x, f->model->d_x + first * sbc::kIn, sizeof(float) * count * sbc::kIn, cudaMemcpyDeviceToHost));
    if (y) CK(cudaMemcpy(y, f->model->d_y + first, sizeof(float) * count, cudaMemcpyDeviceToHost));
    return SBC_OK;
}

int sbc_cost_model_train(sbc_forest* f, int epochs, int batch, double lr, double val_frac, uint64_t seed,
                         sbc_model_stats* st)
{
    if (!f || !f->g || !f->model || epochs < 1 || batch < 128 || batch % 128 || lr <= 0 || val_frac < 0 ||
        val_frac >= 1)
        return fail(SBC_ERR_ARG, "sbc_cost_model_train: bad arguments (log costs first; batch a multiple of 128)");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CostModel* M = f->model;
    cudaStream_t s = f->g->stream;
    CK(cudaStreamSynchronize(s));
    unsigned long long logged = 0;
    CK(cudaMemcpy(&logged, M->d_n, sizeof logged, cudaMemcpyDeviceToHost));
    const int64_t n = std::min<int64_t>((int64_t)logged, M->capacity);
    const int64_t nval = (int64_t)((double)n * val_frac);
    const int64_t ntr = n - nval;
    if (ntr < batch) return fail(SBC_ERR_STATE, "sbc_cost_model_train: %lld logged samples, too few", (long long)n);
    // feature normalisation and the target mean from the training part
    CK(sbc::launch_moments(f, ntr));
    double sums[32];
    CK(cudaMemcpyAsync(sums, M->d_sums, sizeof sums, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    std::vector<float> P(sbc::kModelParams, 0.f);
    std::mt19937_64 rng(seed);
    auto uni = [&](float lim) { return (float)(((double)(rng() >> 11) / 9007199254740992.0) * 2.0 - 1.0) * lim; };
    for (int i = 0; i < sbc::kIn * sbc::kH; ++i) P[sbc::OFF_W1 + i] = uni(std::sqrt(6.f / sbc::kIn));
    for (int i = 0; i < sbc::kH * sbc::kH; ++i) P[sbc::OFF_W2 + i] = uni(std::sqrt(6.f / sbc::kH));
    for (int i = 0; i < sbc::kH; ++i) P[sbc::OFF_W3 + i] = uni(std::sqrt(3.f / sbc::kH));
    const float ymean = (float)(sums[2 * sbc::kIn] / (double)ntr);
    P[sbc::OFF_B3] = ymean;
    for (int k = 0; k < sbc::kIn; ++k) {
        const double mu = sums[k] / (double)ntr;
        const double var = sums[sbc::kIn + k] / (double)ntr - mu * mu;
        P[sbc::OFF_MU + k] = (float)mu;
        P[sbc::OFF_ISD + k] = var > 1e-12 ? (float)(1.0 / std::sqrt(var)) : 1.f;
    }
    CK(cudaMemcpyAsync(M->d_params, P.data(), sizeof(float) * P.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(M->d_m, 0, sizeof(float) * sbc::kTrainParams, s));
    CK(cudaMemsetAsync(M->d_v, 0, sizeof(float) * sbc::kTrainParams, s));
    CK(cudaMemsetAsync(M->d_grad, 0, sizeof(float) * sbc::kTrainParams, s));
    M->adam_t = 0;
    static const int64_t primes[] = {1000003, 2000003, 4000037, 16777259, 104729, 1299709, 15485863, 179424673};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, s));
    const int64_t steps = ntr / batch;
    for (int ep = 0; ep < epochs; ++ep) {
        int64_t mul = 1;
        for (int tries = 0; tries < 64; ++tries) {
            const int64_t p = primes[(rng() >> 7) % (sizeof primes / sizeof primes[0])];
            if (ntr % p) {
                mul = p % ntr ? p : 1;
                break;
            }
        }
        const int64_t add = (int64_t)(rng() % (uint64_t)ntr);
        for (int64_t k = 0; k < steps; ++k) CK(sbc::launch_train_step(f, k * batch, batch, ntr, mul, add, (float)lr));
    }
    CK(cudaEventRecord(e1, s));
    CK(cudaMemsetAsync(M->d_sums, 0, sizeof(double) * 32, s));
    CK(sbc::launch_eval(f, ntr, n, ymean));
    CK(cudaMemcpyAsync(sums, M->d_sums, sizeof sums, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    M->trained = true;
    drop_captured(f);
    if (st) {
        memset(st, 0, sizeof *st);
        st->samples = n;
        st->train_samples = ntr;
        st->val_samples = nval;
        st->epochs = epochs;
        st->steps = steps * epochs;
        st->train_ms = ms;
        if (nval > 0) {
            st->val_mae = sums[24] / (double)nval;
            st->val_rmse = std::sqrt(sums[25] / (double)nval);
            st->val_mae_mean = sums[26] / (double)nval;
        }
    }
    return SBC_OK;
}

int sbc_forest_compare_schedules(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v, int reps,
                                 double* ms_static, double* ms_model)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_forest_compare_schedules: the forest's graph was destroyed");
    if (!f || n <= 0 || !u || !v || reps < 0) return fail(SBC_ERR_ARG, "sbc_forest_compare_schedules: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_forest_compare_schedules before sbc_static_init");
    if (!f->model || !f->model->trained)
        return fail(SBC_ERR_STATE, "sbc_forest_compare_schedules: the cost model is not trained");
    if (n >= INT32_MAX) return fail(SBC_ERR_ARG, "batch too large");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (reps == 0) reps = 1;
    int rc = plan_capacity(g, n, u, v, false);
    if (rc) return rc;
    if ((rc = stage_host(g, n, u, v, false))) return rc;
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    CK(sbc::launch_append(g, (int)n, false));
    TrialState T;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    unsigned long long saved[SBC_NCOUNTERS];
    const bool logging = f->model->logging;
    const int schedule = f->schedule;
    cudaError_t e;
    auto cleanup = [&]() {
        T.release();
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        f->model->logging = logging;
        f->schedule = schedule;
    };
    if ((e = T.alloc(f, f->nk)) || (e = cudaEventCreate(&e0)) || (e = cudaEventCreate(&e1)) ||
        (e = cudaMemcpyAsync(saved, f->d_counters, sizeof saved, cudaMemcpyDeviceToHost, g->stream)) ||
        (e = cudaStreamSynchronize(g->stream))) {
        cleanup();
        return cuda_fail(e, "sbc_forest_compare_schedules setup");
    }
    f->model->logging = false;
    double best[2] = {-1.0, -1.0};
    for (int rep = 0; rep < reps; ++rep) {
        for (int sch = 0; sch < 2; ++sch) {
            f->schedule = sch;
            e = T.copy_from(f, g->stream);
            T.swap(f);
            if (!e) e = cudaEventRecord(e0, g->stream);
            if (!e) e = sbc::launch_update(f, (int)n, false);
            if (!e) e = cudaEventRecord(e1, g->stream);
            T.swap(f);
            if (!e) e = cudaEventSynchronize(e1);
            float t = 0.f;
            if (!e) e = cudaEventElapsedTime(&t, e0, e1);
            if (e) {
                cleanup();
                return cuda_fail(e, "sbc_forest_compare_schedules trial");
            }
            if (best[sch] < 0.0 || t < best[sch]) best[sch] = t;
        }
    }
    cleanup();
    CK(cudaMemcpyAsync(f->d_counters, saved, sizeof saved, cudaMemcpyHostToDevice, g->stream));
    CK(sbc::launch_update(f, (int)n, false));
    CK(sbc::launch_seal(g, (int)n));
    if (ms_static) *ms_static = best[0];
    if (ms_model) *ms_model = best[1];
    return check_graph_err(g);
}

int sbc_set_schedule(sbc_forest* f, int schedule)
{
    if (!f || (schedule != SBC_SCHED_STATIC && schedule != SBC_SCHED_MODEL))
        return fail(SBC_ERR_ARG, "sbc_set_schedule: bad arguments");
    if (schedule == SBC_SCHED_MODEL && (!f->model || !f->model->trained))
        return fail(SBC_ERR_STATE, "sbc_set_schedule: the cost model is not trained");
    if (f->g && use_device(f->g->device)) return SBC_ERR_CUDA;
    if (f->g) CK(cudaStreamSynchronize(f->g->stream));
    f->schedule = schedule;
    drop_captured(f);
    return SBC_OK;
}

int sbc_cost_model_params(sbc_forest* f, float* get, const float* set)
{
    if (!f || !f->g) return fail(SBC_ERR_ARG, "sbc_cost_model_params: null forest or graph");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    int rc = ensure_model(f);
    if (rc) return rc;
    CK(cudaStreamSynchronize(f->g->stream));
    if (set) {
        CK(cudaMemcpy(f->model->d_params, set, sizeof(float) * sbc::kModelParams, cudaMemcpyHostToDevice));
        f->model->trained = true;
        drop_captured(f);
    }
    if (get) CK(cudaMemcpy(get, f->model->d_params, sizeof(float) * sbc::kModelParams, cudaMemcpyDeviceToHost));
    return SBC_OK;
}

int sbc_cost_model_predict(sbc_forest* f, int64_t n, const float* x, float* out)
{
    if (!f || !f->g || !f->model || n < 0 || (n > 0 && (!x || !out)))
        return fail(SBC_ERR_ARG, "sbc_cost_model_predict: bad arguments");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    if (n == 0) return SBC_OK;
    float *dx = nullptr, *dout = nullptr;
    cudaError_t e;
    if ((e = dev_alloc(&dx, (size_t)n * sbc::kIn)) || (e = dev_alloc(&dout, (size_t)n)) ||
        (e = cudaMemcpy(dx, x, sizeof(float) * n * sbc::kIn, cudaMemcpyHostToDevice)) ||
        (e = sbc::launch_predict(f->model->d_params, dx, n, dout, f->g->stream)) ||
        (e = cudaStreamSynchronize(f->g->stream)) ||
        (e = cudaMemcpy(out, dout, sizeof(float) * n, cudaMemcpyDeviceToHost))) {
        dev_free(dx);
        dev_free(dout);
        return cuda_fail(e, "sbc_cost_model_predict");
    }
    dev_free(dx);
    dev_free(dout);
    return SBC_OK;
}

int sbc_cost_model_grad(sbc_forest* f, int64_t n, const float* x, const float* y, float* grad, float* pred)
{
    if (!f || !f->g || !f->model || n <= 0 || n > 65536 || !x || !y || !grad)
        return fail(SBC_ERR_ARG, "sbc_cost_model_grad: bad arguments");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    float *dx = nullptr, *dy = nullptr, *dg = nullptr, *dp = nullptr;
    cudaError_t e;
    cudaStream_t s = f->g->stream;
    if ((e = dev_alloc(&dx, (size_t)n * sbc::kIn)) || (e = dev_alloc(&dy, (size_t)n)) ||
        (e = dev_alloc(&dg, (size_t)sbc::kTrainParams)) || (e = dev_alloc(&dp, (size_t)n)) ||
        (e = cudaMemcpy(dx, x, sizeof(float) * n * sbc::kIn, cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice)) ||
        (e = cudaMemsetAsync(dg, 0, sizeof(float) * sbc::kTrainParams, s)) ||
        (e = sbc::launch_grad(f->model->d_params, dg, dx, dy, 0, n, n, 1, 0, dp, s)) ||
        (e = cudaStreamSynchronize(s)) ||
        (e = cudaMemcpy(grad, dg, sizeof(float) * sbc::kTrainParams, cudaMemcpyDeviceToHost)) ||
        (pred && (e = cudaMemcpy(pred, dp, sizeof(float) * n, cudaMemcpyDeviceToHost)))) {
        dev_free(dx), dev_free(dy), dev_free(dg), dev_free(dp);
        return cuda_fail(e, "sbc_cost_model_grad");
    }
    dev_free(dx), dev_free(dy), dev_free(dg), dev_free(dp);
    return SBC_OK;
}

int sbc_get_roster(sbc_forest* f, int64_t r, int level, int32_t* out, int* n)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "state read: the forest's graph was destroyed");
    if (!f || !n || r < 0 || r >= f->nk || level < 0 || level >= sbc::kRosterLevels)
        return fail(SBC_ERR_ARG, "sbc_get_roster: bad arguments");
    if (!f->d_roster) {
        *n = -1;
        return SBC_OK;
    }
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaStreamSynchronize(f->g->stream));
    const size_t w = (size_t)r * sbc::kRosterLevels + level;
    int c = 0;
    CK(cudaMemcpy(&c, f->d_roster_n + w, sizeof c, cudaMemcpyDeviceToHost));
    *n = c <= sbc::kRosterCap ? c : -1;
    if (out && c > 0 && c <= sbc::kRosterCap)
        CK(cudaMemcpy(out, f->d_roster + w * sbc::kRosterCap, sizeof(int32_t) * c, cudaMemcpyDeviceToHost));
    return SBC_OK;
}

int sbc_get_level_hist(sbc_forest* f, int64_t r0, int64_t nr, int32_t* out)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "state read: the forest's graph was destroyed");
    if (!f || !out || r0 < 0 || nr < 0 || r0 + nr > f->nk) return fail(SBC_ERR_ARG, "level hist: bad row range");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaMemcpyAsync(out, f->d_lvlhist + r0 * sbc::kHistLevels, sizeof(int32_t) * nr * sbc::kHistLevels,
                       cudaMemcpyDeviceToHost, f->g->stream));
    CK(cudaStreamSynchronize(f->g->stream));
    return SBC_OK;
}

// ------------------------------------------------------------------ groups

int sbc_group_create(sbc_group** out, int n, sbc_forest* const* forests, int variant)
{
    if (!out || n < 1 || !forests) return fail(SBC_ERR_ARG, "sbc_group_create: bad arguments");
    *out = nullptr;
    if (n > sbc::kMaxGroup) return fail(SBC_ERR_ARG, "sbc_group_create: at most %d forests", sbc::kMaxGroup);
    if (variant >= sbc::group_variant_count()) return fail(SBC_ERR_ARG, "update variant %d out of range", variant);
    int64_t total = 0, nv_max = 0;
    for (int i = 0; i < n; ++i) {
        sbc_forest* f = forests[i];
        if (!f || !f->g) return fail(SBC_ERR_ARG, "sbc_group_create: forest %d is null or lost its graph", i);
        if (f->device != forests[0]->device) return fail(SBC_ERR_ARG, "sbc_group_create: forests on different devices");
        for (int j = 0; j < i; ++j)
            if (forests[j] == f || forests[j]->g == f->g)
                return fail(SBC_ERR_ARG, "sbc_group_create: forests %d and %d share a forest or a graph", j, i);
        if (f->nk >= (int64_t)1 << 25) return fail(SBC_ERR_ARG, "sbc_group_create: forest %d has too many roots", i);
        total += f->nk;
        nv_max = std::max<int64_t>(nv_max, f->nv);
    }
    if (total >= INT32_MAX) return fail(SBC_ERR_ARG, "sbc_group_create: too many roots in total");
    if (use_device(forests[0]->device)) return SBC_ERR_CUDA;
    sbc_group* G = new sbc_group();
    G->device = forests[0]->device;
    G->nv_max = nv_max;
    G->total_roots = total;
    G->sm_count = forests[0]->sm_count;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
        return forests[a]->nk * forests[a]->nv > forests[b]->nk * forests[b]->nv;
    });
    for (int s = 0; s < n; ++s) {
        G->order.push_back(idx[s]);
        G->members.push_back(forests[idx[s]]);
    }
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking)) ||
        (e = cudaEventCreateWithFlags(&G->ev, cudaEventDisableTiming)) || (e = cudaEventCreate(&G->t0)) ||
        (e = cudaEventCreate(&G->t1)) || (e = dev_alloc(&G->d_worklist, (size_t)total)) ||
        (e = dev_alloc(&G->d_nwork, 2)) || (e = dev_alloc(&G->d_counters, SBC_NCOUNTERS)) ||
        (e = dev_alloc(&G->d_errs, sbc::kMaxGroup)) ||
        (e = cudaMallocHost((void**)&G->h_errs, sizeof(int) * sbc::kMaxGroup)) ||
        (e = cudaMemsetAsync(G->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, G->stream))) {
        sbc_group_destroy(G);
        return cuda_fail(e, "sbc_group_create");
    }
    if (variant < 0) variant = nv_max <= 8192 ? 3 : (nv_max <= 262144 ? 5 : sbc::update_default_variant());
    int rc = group_alloc_scratch(G, variant);
    if (rc) {
        sbc_group_destroy(G);
        return rc;
    }
    CK(cudaStreamSynchronize(G->stream));
    for (sbc_forest* f : G->members) f->groups++;
    *out = G;
    return SBC_OK;
}

int sbc_group_destroy(sbc_group* G)
{
    if (!G) return SBC_OK;
    use_device(G->device);
    if (G->stream) cudaStreamSynchronize(G->stream);
    for (sbc_forest* f : G->members) f->groups--;
    group_free_scratch(G);
    dev_free(G->d_worklist);
    dev_free(G->d_nwork);
    dev_free(G->d_counters);
    dev_free(G->d_errs);
    if (G->h_errs) cudaFreeHost(G->h_errs);
    if (G->ev) cudaEventDestroy(G->ev);
    if (G->t0) cudaEventDestroy(G->t0);
    if (G->t1) cudaEventDestroy(G->t1);
    if (G->h_bc) cudaFreeHost(G->h_bc);
    if (G->stream) cudaStreamDestroy(G->stream);
    delete G;
    return SBC_OK;
}

int sbc_group_get_bc(sbc_group* G, double* bc)
{
    int rc = group_check(G);
    if (rc) return rc;
    if (!bc) return fail(SBC_ERR_ARG, "sbc_group_get_bc: null");
    if ((rc = group_after_members(G))) return rc;
    int64_t total = 0;
    for (sbc_forest* f : G->members) total += f->nv;
    if (total > G->h_bc_cap) {
        if (G->h_bc) cudaFreeHost(G->h_bc);
        G->h_bc = nullptr;
        G->h_bc_cap = 0;
        CK(cudaMallocHost(&G->h_bc, sizeof(double) * std::max<int64_t>(total, 1)));
        G->h_bc_cap = total;
    }
    // one asynchronous copy per member into pinned memory, one wait; slot s
    // holds the caller's member order[s], whose vector goes at its offset in
    // the caller's order
    const size_t n = G->members.size();
    std::vector<int64_t> at(n + 1, 0);
    for (size_t s = 0; s < n; ++s) at[G->order[s] + 1] = G->members[s]->nv;
    for (size_t i = 0; i < n; ++i) at[i + 1] += at[i];
    for (size_t s = 0; s < n; ++s) {
        sbc_forest* f = G->members[s];
        CK(cudaMemcpyAsync(G->h_bc + at[G->order[s]], f->d_bc, sizeof(double) * f->nv, cudaMemcpyDeviceToHost,
                           G->stream));
    }
    CK(cudaStreamSynchronize(G->stream));
    memcpy(bc, G->h_bc, sizeof(double) * total);
    return SBC_OK;
}

int sbc_group_info(const sbc_group* G, int* n, int64_t* workers, int64_t* bytes, int* variant)
{
    if (!G) return fail(SBC_ERR_ARG, "sbc_group_info: null");
    if (n) *n = (int)G->members.size();
    if (workers) *workers = G->ws.workers;
    if (bytes) *bytes = (int64_t)G->ws.bytes() + G->total_roots * 4;
    if (variant) *variant = G->variant;
    return SBC_OK;
}

int sbc_group_set_variant(sbc_group* G, int variant)
{
    int rc = group_check(G);
    if (rc) return rc;
    if (variant < 0 || variant >= sbc::group_variant_count())
        return fail(SBC_ERR_ARG, "update variant %d out of range", variant);
    CK(cudaStreamSynchronize(G->stream));
    if ((rc = group_alloc_scratch(G, variant))) return rc;
    CK(cudaStreamSynchronize(G->stream));
    return SBC_OK;
}

int sbc_group_insert_batch(sbc_group* G, const int64_t* counts, const int64_t* u, const int64_t* v, double* device_ms)
{
    int rc = group_check(G);
    if (rc) return rc;
    if (!counts) return fail(SBC_ERR_ARG, "sbc_group_insert_batch: null counts");
    for (sbc_forest* f : G->members)
        if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_group_insert_batch before sbc_static_init of a member");
    std::vector<int> cs;
    if ((rc = group_stage(G, counts, u, v, cs))) return rc;
    if ((rc = group_after_members(G))) return rc;
    const int ns = (int)G->members.size();
    CK(cudaMemsetAsync(G->d_errs, 0, sizeof(int) * ns, G->stream));
    CK(cudaEventRecord(G->t0, G->stream));
    CK(sbc::launch_group_update(G, cs.data(), sbc::GROUP_ALL));
    CK(cudaEventRecord(G->t1, G->stream));
    // every member's slack error flag, gathered by the seal: one copy
    CK(cudaMemcpyAsync(G->h_errs, G->d_errs, sizeof(int) * ns, cudaMemcpyDeviceToHost, G->stream));
    if ((rc = members_after_group(G))) return rc;
    CK(cudaStreamSynchronize(G->stream));
    if (device_ms) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, G->t0, G->t1));
        *device_ms = t;
    }
    for (int s = 0; s < ns; ++s)
        if (G->h_errs[s]) {
            sbc_graph* g = G->members[s]->g;
            cudaMemsetAsync(g->d_err, 0, sizeof(int), g->stream);
            return fail(SBC_ERR_STATE, "adjacency slack exhausted during an insertion batch (reserve capacity first)");
        }
    return SBC_OK;
}

int sbc_group_autotune(sbc_group* G, const int64_t* counts, const int64_t* u, const int64_t* v, int reps, int* chosen,
                       double* ms, int ms_len)
{
    int rc = group_check(G);
    if (rc) return rc;
    if (!counts || reps < 0 || ms_len < 0 || (ms_len > 0 && !ms))
        return fail(SBC_ERR_ARG, "sbc_group_autotune: bad arguments");
    for (sbc_forest* f : G->members)
        if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_group_autotune before sbc_static_init of a member");
    if (reps == 0) reps = 2;
    for (int i = 0; i < ms_len; ++i) ms[i] = -1.0;
    std::vector<int> cs;
    if ((rc = group_stage(G, counts, u, v, cs))) return rc;
    if ((rc = group_after_members(G))) return rc;
    CK(sbc::launch_group_update(G, cs.data(), sbc::GROUP_APPEND));
    CK(cudaStreamSynchronize(G->stream));
    // trial copies of every member's full state
    const int ns = (int)G->members.size();
    std::vector<TrialState> T(ns);
    size_t need = 0, free_b = 0, total_b = 0;
    for (sbc_forest* f : G->members) need += (size_t)f->nk * (size_t)f->nv * 21 + (size_t)f->nv * 8;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const bool can_time = need <= free_b / 2;
    unsigned long long saved[SBC_NCOUNTERS];
    CK(cudaMemcpy(saved, G->d_counters, sizeof saved, cudaMemcpyDeviceToHost));
    int best = G->variant;
    double best_ms = -1.0;
    cudaError_t e = cudaSuccess;
    auto release = [&]() {
        for (auto& t : T) t.release();
    };
    for (int s = 0; can_time && s < ns && !e; ++s) e = T[s].alloc(G->members[s], G->members[s]->nk);
    if (e) {
        release();
        return cuda_fail(e, "sbc_group_autotune trial copies");
    }
    for (int c = 0; can_time && c < sbc::group_variant_count(); ++c) {
        CK(cudaMemGetInfo(&free_b, &total_b));
        const int per_sm = std::max(1, sbc::group_workers_per_sm(c));
        const int64_t want = std::min<int64_t>((int64_t)per_sm * G->sm_count, G->total_roots);
        if ((size_t)want * WorkerScratch::per_worker(G->nv_max) > (free_b + G->ws.bytes()) / 2) continue;
        if ((rc = group_alloc_scratch(G, c))) {
            release();
            return rc;
        }
        double c_ms = -1.0;
        for (int rep = 0; rep < reps; ++rep) {
            for (int s = 0; s < ns && !e; ++s) e = T[s].copy_from(G->members[s], G->stream);
            for (int s = 0; s < ns; ++s) T[s].swap(G->members[s]);
            if (!e) e = cudaEventRecord(G->t0, G->stream);
            if (!e) e = sbc::launch_group_update(G, cs.data(), sbc::GROUP_UPDATE);
            if (!e) e = cudaEventRecord(G->t1, G->stream);
            for (int s = 0; s < ns; ++s) T[s].swap(G->members[s]);
            if (!e) e = cudaEventSynchronize(G->t1);
            float t = 0.f;
            if (!e) e = cudaEventElapsedTime(&t, G->t0, G->t1);
            if (e) {
                release();
                return cuda_fail(e, "sbc_group_autotune trial");
            }
            if (c_ms < 0.0 || t < c_ms) c_ms = t;
        }
        if (c < ms_len) ms[c] = c_ms;
        if (best_ms < 0.0 || c_ms < best_ms) {
            best = c;
            best_ms = c_ms;
        }
    }
    release();
    if (best != G->variant && (rc = group_alloc_scratch(G, best))) return rc;
    CK(cudaMemcpyAsync(G->d_counters, saved, sizeof saved, cudaMemcpyHostToDevice, G->stream));
    CK(sbc::launch_group_update(G, cs.data(), sbc::GROUP_UPDATE | sbc::GROUP_SEAL));
    if ((rc = members_after_group(G))) return rc;
    CK(cudaStreamSynchronize(G->stream));
    if (chosen) *chosen = best;
    for (sbc_forest* f : G->members)
        if ((rc = check_graph_err(f->g))) return rc;
    return SBC_OK;
}

int sbc_group_read_counters(sbc_group* G, int64_t* vertices, int64_t* edges, int64_t* case1, int64_t* case2,
                            int64_t* scanned)
{
    int rc = group_check(G);
    if (rc) return rc;
    unsigned long long c[SBC_NCOUNTERS];
    CK(cudaMemcpyAsync(c, G->d_counters, sizeof c, cudaMemcpyDeviceToHost, G->stream));
    CK(cudaMemsetAsync(G->d_counters, 0, sizeof c, G->stream));
    CK(cudaStreamSynchronize(G->stream));
    if (vertices) *vertices = (int64_t)c[0];
    if (edges) *edges = (int64_t)c[1];
    if (case1) *case1 = (int64_t)c[2];
    if (case2) *case2 = (int64_t)c[3];
    if (scanned) *scanned = (int64_t)c[4];
    return SBC_OK;
}

int sbc_update_inserted(sbc_forest* f, int64_t n, const int64_t* u, const int64_t* v, sbc_batch_stats* stats)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_update_inserted: the forest's graph was destroyed");
    if (!f || n < 0 || (n > 0 && (!u || !v))) return fail(SBC_ERR_ARG, "sbc_update_inserted: bad arguments");
    if (!f->initialized) return fail(SBC_ERR_STATE, "sbc_update_inserted before sbc_static_init");
    sbc_graph* g = f->g;
    if (use_device(g->device)) return SBC_ERR_CUDA;
    if (n == 0) {
        if (stats) memset(stats, 0, sizeof *stats);
        return SBC_OK;
    }
    int rc = stage_host(g, n, u, v, true);
    if (rc) return rc;
    if ((rc = ensure_model_batch(f, g->ins_capacity))) return rc;
    if (stats) CK(cudaMemsetAsync(f->d_counters, 0, sizeof(unsigned long long) * SBC_NCOUNTERS, g->stream));
    f->prof_begin(sbc::PROF_BATCH);
    CK(sbc::launch_update(f, (int)n, true));
    f->prof_end(sbc::PROF_BATCH);
    if (stats) return collect_stats(f, n, stats);
    CK(cudaStreamSynchronize(g->stream));
    return SBC_OK;
}

int sbc_sync(sbc_forest* f)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_sync: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_sync: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaStreamSynchronize(f->g->stream));
    return check_graph_err(f->g);
}

int sbc_read_counters(sbc_forest* f, int64_t* vertices, int64_t* edges, int64_t* case1, int64_t* case2,
                      int64_t* scanned)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_read_counters: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_read_counters: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    unsigned long long c[SBC_NCOUNTERS];
    CK(cudaMemcpyAsync(c, f->d_counters, sizeof c, cudaMemcpyDeviceToHost, f->g->stream));
    CK(cudaMemsetAsync(f->d_counters, 0, sizeof c, f->g->stream));
    CK(cudaStreamSynchronize(f->g->stream));
    if (vertices) *vertices = (int64_t)c[0];
    if (edges) *edges = (int64_t)c[1];
    if (case1) *case1 = (int64_t)c[2];
    if (case2) *case2 = (int64_t)c[3];
    if (scanned) *scanned = (int64_t)c[4];
    return SBC_OK;
}

int sbc_get_bc(sbc_forest* f, double* out)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_get_bc: the forest's graph was destroyed");
    if (!f || !out) return fail(SBC_ERR_ARG, "sbc_get_bc: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaMemcpyAsync(out, f->d_bc, sizeof(double) * f->nv, cudaMemcpyDeviceToHost, f->g->stream));
    CK(cudaStreamSynchronize(f->g->stream));
    return SBC_OK;
}

int sbc_get_dist(sbc_forest* f, int64_t r0, int64_t nr, int32_t* out) { return get_rows(f, f ? f->d_dist : nullptr, r0, nr, out); }
int sbc_get_sigma(sbc_forest* f, int64_t r0, int64_t nr, int64_t* out) { return get_rows(f, f ? f->d_sigma : nullptr, r0, nr, out); }
int sbc_get_delta(sbc_forest* f, int64_t r0, int64_t nr, double* out) { return get_rows(f, f ? f->d_delta : nullptr, r0, nr, out); }

int sbc_set_profiling(sbc_forest* f, int on)
{
    if (!f) return fail(SBC_ERR_ARG, "sbc_set_profiling: null");
    f->prof = on != 0;
    return SBC_OK;
}

int sbc_get_profile(sbc_forest* f, sbc_profile* out)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_get_profile: the forest's graph was destroyed");
    if (!f || !out) return fail(SBC_ERR_ARG, "sbc_get_profile: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    for (int k = 0; k < sbc::PROF_COUNT; ++k) f->prof_collect(k);
    out->static_ms = f->prof_ms[sbc::PROF_STATIC];
    out->static_launches = f->prof_n[sbc::PROF_STATIC];
    out->append_ms = f->prof_ms[sbc::PROF_APPEND];
    out->append_launches = f->prof_n[sbc::PROF_APPEND];
    out->classify_ms = f->prof_ms[sbc::PROF_CLASSIFY];
    out->classify_launches = f->prof_n[sbc::PROF_CLASSIFY];
    out->update_ms = f->prof_ms[sbc::PROF_UPDATE];
    out->update_launches = f->prof_n[sbc::PROF_UPDATE];
    out->batch_ms = f->prof_ms[sbc::PROF_BATCH];
    out->batches = f->prof_n[sbc::PROF_BATCH];
    return SBC_OK;
}

int sbc_reset_profile(sbc_forest* f)
{
    if (!f) return fail(SBC_ERR_ARG, "sbc_reset_profile: null");
    for (int k = 0; k < sbc::PROF_COUNT; ++k) {
        f->prof_collect(k);
        f->prof_ms[k] = 0;
        f->prof_n[k] = 0;
    }
    return SBC_OK;
}

int sbc_timer_start(sbc_forest* f)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_timer_start: the forest's graph was destroyed");
    if (!f) return fail(SBC_ERR_ARG, "sbc_timer_start: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaEventRecord(f->t0, f->g->stream));
    return SBC_OK;
}

int sbc_timer_stop(sbc_forest* f, double* ms)
{
    if (f && !f->g) return fail(SBC_ERR_STATE, "sbc_timer_stop: the forest's graph was destroyed");
    if (!f || !ms) return fail(SBC_ERR_ARG, "sbc_timer_stop: null");
    if (use_device(f->g->device)) return SBC_ERR_CUDA;
    CK(cudaEventRecord(f->t1, f->g->stream));
    CK(cudaEventSynchronize(f->t1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, f->t0, f->t1));
    *ms = t;
    return SBC_OK;
}

// ============================================================ STINGER shim

struct stinger {
    sbc_graph* g;
};

struct stinger* stinger_new(void)
{
    stinger* s = (stinger*)calloc(1, sizeof(stinger));
    return s;
}

void stinger_set_initial_edges(struct stinger* G, const size_t nv, const int64_t etype, const int64_t* off,
                               const int64_t* phys_to, const int64_t* weights, const int64_t* times,
                               const int64_t* first_times, const int64_t single_ts)
{
    (void)etype;
    (void)weights;
    (void)times;
    (void)first_times;
    (void)single_ts;
    if (!G) {
        fail(SBC_ERR_ARG, "stinger_set_initial_edges: null graph");
        return;
    }
    if (G->g) {
        sbc_graph_destroy(G->g);
        G->g = nullptr;
    }
    sbc_graph_create(&G->g, (int64_t)nv, off, phys_to);
}

int stinger_insert_edge(struct stinger* G, int64_t type, int64_t from, int64_t to, int64_t weight, int64_t timestamp)
{
    (void)type;
    (void)weight;
    (void)timestamp;
    if (!G || !G->g) return -1;
    int result = -1;
    if (sbc_graph_insert_directed(G->g, from, to, &result)) return -1;
    return result;
}

int stinger_insert_edge_pair(struct stinger* G, int64_t type, int64_t from, int64_t to, int64_t weight,
                             int64_t timestamp)
{
    int a = stinger_insert_edge(G, type, from, to, weight, timestamp);
    int b = stinger_insert_edge(G, type, to, from, weight, timestamp);
    if (a < 0 || b < 0) return -1;
    return a | b;
}

int stinger_remove_edge(struct stinger* G, int64_t type, int64_t from, int64_t to)
{
    (void)type;
    if (!G || !G->g) return -1;
    int res = -1;
    if (sbc_graph_remove_directed(G->g, from, to, &res)) return -1;
    return res == 1 ? 1 : -1;  // an absent edge falls through to -1 (src/stinger/stinger.c:1089)
}

int64_t stinger_outdegree(const struct stinger* G, int64_t v)
{
    if (!G || !G->g) return 0;
    int64_t d = 0;
    if (sbc_graph_degree(G->g, v, &d)) return 0;
    return d;
}

int64_t stinger_typed_outdegree(const struct stinger* G, int64_t v, int64_t type)
{
    (void)type;
    return stinger_outdegree(G, v);
}

struct stinger* stinger_free(struct stinger* G)
{
    if (G) {
        sbc_graph_destroy(G->g);
        free(G);
    }
    return nullptr;
}

struct sbc_graph* stinger_sbc_graph(struct stinger* G) { return G ? G->g : nullptr; }

// ======================================================= streamingbc.h surface

static bcForest* make_host_forest(int64_t NV, int64_t NK, const int64_t* roots)
{
    bcForest* f = (bcForest*)calloc(1, sizeof(bcForest));
    if (!f) return nullptr;
    f->NV = NV;
    f->forest = (bcTreePtr*)calloc((size_t)(NV > 0 ? NV : 1), sizeof(bcTreePtr));
    f->totalBC = (bc_t*)calloc((size_t)(NV > 0 ? NV : 1), sizeof(bc_t));
    f->sbc_nk = NK;
    f->sbc_roots = (int64_t*)malloc(sizeof(int64_t) * (size_t)(NK > 0 ? NK : 1));
    if (!f->forest || !f->totalBC || !f->sbc_roots) {
        free(f->forest);
        free(f->totalBC);
        free(f->sbc_roots);
        free(f);
        return nullptr;
    }
    for (int64_t r = 0; r < NK; ++r) f->sbc_roots[r] = roots ? roots[r] : r;
    return f;
}

bcForest* streamingBCCreateForestExact(int64_t NV) { return make_host_forest(NV, NV, nullptr); }

bcForest* streamingBCCreateForestApproximate(int64_t NV, int64_t NK, int64_t* rootArrayForApproximation)
{
    if (NK > NV || NK < 0 || !rootArrayForApproximation) {
        fail(SBC_ERR_ARG, "streamingBCCreateForestApproximate: bad arguments");
        return nullptr;
    }
    return make_host_forest(NV, NK, rootArrayForApproximation);
}

static void free_host_forest(bcForestPtr* dead)
{
    if (!dead || !*dead) return;
    bcForest* f = *dead;
    for (int64_t v = 0; v < f->NV; ++v)
        if (f->forest[v]) {
            free(f->forest[v]->vArr);
            free(f->forest[v]);
        }
    sbc_forest_destroy(f->sbc);
    free(f->forest);
    free(f->totalBC);
    free(f->sbc_roots);
    free(f);
    *dead = nullptr;
}

void streamingBCDeleteForestExact(bcForestPtr* deadForest) { free_host_forest(deadForest); }

void streamingBCDeleteForestApproximate(bcForestPtr* deadForest, int64_t rootArraySize, int64_t* rootArray)
{
    (void)rootArraySize;
    (void)rootArray;
    free_host_forest(deadForest);
}

extraArraysPerThread** streamingBCCreateAuxilary(int64_t threadCount, int64_t NV)
{
    (void)NV;
    if (threadCount < 1) threadCount = 1;
    extraArraysPerThread** a = (extraArraysPerThread**)calloc((size_t)threadCount, sizeof(extraArraysPerThread*));
    if (!a) return nullptr;
    for (int64_t t = 0; t < threadCount; ++t) a[t] = (extraArraysPerThread*)calloc(1, sizeof(extraArraysPerThread));
    return a;
}

void streamingBCDeleteAuxilary(extraArraysPerThread** parallelExtra, int64_t threadCount, int64_t NV)
{
    (void)NV;
    if (!parallelExtra) return;
    for (int64_t t = 0; t < threadCount; ++t) free(parallelExtra[t]);
    free(parallelExtra);
}

void ClearCounters(extraArraysPerThread* eapt)
{
    if (eapt) memset(eapt, 0, sizeof *eapt);
}

static int refresh_bc(bcForest* forest) { return sbc_get_bc(forest->sbc, forest->totalBC); }

static void static_common(bcForest* forest, struct stinger* G, extraArraysPerThread** aux)
{
    if (!forest || !G || !G->g) {
        fail(SBC_ERR_ARG, "streamingBCInitStatic: forest or graph missing");
        return;
    }
    if (forest->sbc && forest->sbc->g != G->g) {
        sbc_forest_destroy(forest->sbc);
        forest->sbc = nullptr;
    }
    if (!forest->sbc && sbc_forest_create(&forest->sbc, G->g, forest->sbc_nk, forest->sbc_roots, 0)) return;
    if (sbc_static_init(forest->sbc)) return;
    int64_t vtx = 0, edg = 0;
    if (sbc_read_counters(forest->sbc, &vtx, &edg, nullptr, nullptr, nullptr)) return;
    if (aux && aux[0]) {
        aux[0]->staticTraverseVerticeCounter += vtx;
        aux[0]->staticTraverseEdgeCounter += edg;
    }
    refresh_bc(forest);
}

void streamingBCInitStaticExact(bcForest* forest, struct stinger* stingerGraph, int64_t NT,
                                extraArraysPerThread** auxilary)
{
    (void)NT;
    static_common(forest, stingerGraph, auxilary);
}

void streamingBCInitStaticApproximate(bcForest* forest, struct stinger* stingerGraph, int64_t NT,
                                      extraArraysPerThread** auxilary, int64_t NK, int64_t* rootArrayForApproximation)
{
    (void)NT;
    if (forest && rootArrayForApproximation && NK == forest->sbc_nk)
        memcpy(forest->sbc_roots, rootArrayForApproximation, sizeof(int64_t) * (size_t)NK);
    static_common(forest, stingerGraph, auxilary);
}

StreamingExtraInfo insertEdgeStreamingBC(bcForest* forest, struct stinger* sStinger, int64_t newU, int64_t newV,
                                         int64_t* rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                         extraArraysPerThread** eAPT, uint32_t loadBalancing, uint32_t granularity)
{
    (void)rootArrayForApproximation;
    (void)NV;
    (void)NT;
    (void)loadBalancing;
    (void)granularity;
    StreamingExtraInfo sei = {0, 0, 0, 0};
    if (!forest || !forest->sbc || !sStinger || forest->sbc->g != sStinger->g) {
        fail(SBC_ERR_STATE, "insertEdgeStreamingBC: static init on this graph has not run");
        return sei;
    }
    sbc_batch_stats st;
    if (sbc_update_inserted(forest->sbc, 1, &newU, &newV, &st)) return sei;
    sei.adjacent = st.case1;
    sei.movement = st.case2;
    sei.sameLevel = NK - st.case1 - st.case2;
    if (eAPT && eAPT[0]) {
        eAPT[0]->adjacentCounter += st.case1;
        eAPT[0]->movementCounter += st.case2;
        eAPT[0]->dynamicTraverseVerticeCounter += st.vertices;
        eAPT[0]->dynamicTraverseEdgeCounter += st.edges;
    }
    refresh_bc(forest);
    return sei;
}

StreamingExtraInfo deleteEdgeStreamingBC(bcForest* forest, struct stinger* sStinger, int64_t oldU, int64_t oldV,
                                         int64_t* rootArrayForApproximation, int64_t NK, int64_t Nv, int64_t NT,
                                         extraArraysPerThread** eAPT, uint32_t loadBalancing, uint32_t granularity)
{
    // The caller has already removed (oldU, oldV) in both directions
    // (stinger_remove_edge x2, src/sbcMain_utils.c:477-484).
    (void)rootArrayForApproximation;
    (void)Nv;
    (void)NT;
    (void)loadBalancing;
    (void)granularity;
    StreamingExtraInfo sei = {0, 0, 0, 0};
    if (!forest || !forest->sbc || !sStinger || forest->sbc->g != sStinger->g) {
        fail(SBC_ERR_STATE, "deleteEdgeStreamingBC: static init on this graph has not run");
        return sei;
    }
    sbc_batch_stats st;
    if (sbc_update_deleted(forest->sbc, oldU, oldV, &st)) return sei;
    sei.adjacent = st.case1;
    sei.movement = st.case2;
    sei.sameLevel = NK - st.case1 - st.case2;
    if (eAPT && eAPT[0]) {
        eAPT[0]->adjacentCounter += st.case1;
        eAPT[0]->movementCounter += st.case2;
        eAPT[0]->dynamicTraverseVerticeCounter += st.vertices;
        eAPT[0]->dynamicTraverseEdgeCounter += st.edges;
    }
    refresh_bc(forest);
    return sei;
}

// src/streamingbc.c:56-77: the reference inserts the vertex's edges (src,
// adjacencyArray[d]) into the graph and updates the forest one edge at a
// time.  Here all of them go to the device as one batch (sbc_insert_batch):
// appended in array order, each applied to every root in that order, so the
// state is the one the edge-by-edge loop reaches, in one append, one
// classify and one update launch instead of one synchronous call per edge.
// An entry that is already an edge, repeats an earlier entry, is src itself
// or lies outside the graph is skipped (the reference would apply the update
// of an existing edge a second time).
StreamingExtraInfo insertVertexStreamingBC(bcForest* forest, struct stinger* sStinger, int64_t src,
                                           int64_t* adjacencyArray, int64_t adjacencySize,
                                           int64_t* rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                           extraArraysPerThread** eAPT)
{
    (void)rootArrayForApproximation;
    (void)NV;
    (void)NT;
    StreamingExtraInfo total = {0, 0, 0, 0};
    if (!forest || !forest->sbc || !sStinger || forest->sbc->g != sStinger->g) {
        fail(SBC_ERR_STATE, "insertVertexStreamingBC: static init on this graph has not run");
        return total;
    }
    if (adjacencySize <= 0) return total;
    if (!adjacencyArray) {
        fail(SBC_ERR_ARG, "insertVertexStreamingBC: null adjacency array");
        return total;
    }
    std::vector<int64_t> us((size_t)adjacencySize, src);
    sbc_batch_stats st;
    if (sbc_insert_batch(forest->sbc, adjacencySize, us.data(), adjacencyArray, &st)) return total;
    total.adjacent = st.case1;
    total.movement = st.case2;
    total.sameLevel = NK * st.inserted - st.case1 - st.case2;
    if (eAPT && eAPT[0]) {
        eAPT[0]->adjacentCounter += st.case1;
        eAPT[0]->movementCounter += st.case2;
        eAPT[0]->dynamicTraverseVerticeCounter += st.vertices;
        eAPT[0]->dynamicTraverseEdgeCounter += st.edges;
    }
    refresh_bc(forest);
    return total;
}

// src/streamingbc.c:229-256: remove every edge of src, one at a time, each
// followed by deleteEdgeStreamingBC.  adjacencyArray receives the former
// neighbours and *adjacencySize their number (the reference intends this but
// never advances its index, so it reports 0).
StreamingExtraInfo deleteVertexStreamingBC(bcForest* forest, struct stinger* sStinger, int64_t src,
                                           int64_t* adjacencyArray, int64_t* adjacencySize,
                                           int64_t* rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                           extraArraysPerThread** eAPT)
{
    StreamingExtraInfo total = {0, 0, 0, 0};
    if (adjacencySize) *adjacencySize = 0;
    if (!sStinger || !sStinger->g) {
        fail(SBC_ERR_STATE, "deleteVertexStreamingBC: no graph");
        return total;
    }
    int64_t n = 0;
    if (sbc_graph_neighbors(sStinger->g, src, nullptr, 0, &n)) return total;
    std::vector<int64_t> nbr((size_t)n);
    if (n && sbc_graph_neighbors(sStinger->g, src, nbr.data(), n, &n)) return total;
    for (int64_t d = 0; d < n; ++d) {
        const int64_t dest = nbr[d];
        if (adjacencyArray) adjacencyArray[d] = dest;
        stinger_remove_edge(sStinger, 0, src, dest);
        stinger_remove_edge(sStinger, 0, dest, src);
        StreamingExtraInfo one = deleteEdgeStreamingBC(forest, sStinger, src, dest, rootArrayForApproximation, NK, NV,
                                                       NT, eAPT, BALANCE, FINE);
        total.adjacent += one.adjacent;
        total.movement += one.movement;
        total.sameLevel += one.sameLevel;
    }
    if (adjacencySize) *adjacencySize = n;
    return total;
}

int streamingBCSyncForest(bcForest* forest)
{
    if (!forest || !forest->sbc) return fail(SBC_ERR_STATE, "streamingBCSyncForest: no device forest");
    sbc_forest* f = forest->sbc;
    const int64_t nv = forest->NV;
    std::vector<int32_t> dist(nv);
    std::vector<int64_t> sig(nv);
    std::vector<double> del(nv);
    for (int64_t r = 0; r < f->nk; ++r) {
        int rc;
        if ((rc = sbc_get_dist(f, r, 1, dist.data())) || (rc = sbc_get_sigma(f, r, 1, sig.data())) ||
            (rc = sbc_get_delta(f, r, 1, del.data())))
            return rc;
        const int64_t root = f->h_roots[r];
        bcTree* t = forest->forest[root];
        if (!t) {
            t = (bcTree*)calloc(1, sizeof(bcTree));
            if (!t) return fail(SBC_ERR_NOMEM, "streamingBCSyncForest: host allocation");
            t->NV = nv;
            t->vArr = (bcV*)calloc((size_t)(nv > 0 ? nv : 1), sizeof(bcV));
            if (!t->vArr) {
                free(t);
                return fail(SBC_ERR_NOMEM, "streamingBCSyncForest: host allocation");
            }
            forest->forest[root] = t;
        }
        for (int64_t x = 0; x < nv; ++x) {
            const bool reach = dist[x] != SBC_INF;
            t->vArr[x].level = reach ? dist[x] : INT64_MAX;
            t->vArr[x].sigma = reach ? sig[x] : INT64_MAX;
            t->vArr[x].delta = del[x];
            t->vArr[x].edgesAbove = 0;
            t->vArr[x].edgesBelow = 0;
        }
    }
    return refresh_bc(forest);
}

// ---- CSR helpers of the reference driver (src/sbcMain_utils.c:306-362, :425-456)

void CreateStingerFromCSR(csrGraph* csr, struct stinger** stingerGraph)
{
    if (!csr || !stingerGraph) return;
    *stingerGraph = stinger_new();
    stinger_set_initial_edges(*stingerGraph, (size_t)csr->NV, 0, csr->vertexPointerArray, csr->edgeArray, nullptr,
                              nullptr, nullptr, 0);
}

static csrGraph* empty_csr(int64_t NV, int64_t NE)
{
    csrGraph* g = (csrGraph*)malloc(sizeof(csrGraph));
    if (!g) return nullptr;
    g->NV = NV;
    g->NE = NE;
    g->vertexPointerArray = (int64_t*)calloc((size_t)NV + 1, sizeof(int64_t));
    g->edgeArray = (int64_t*)malloc(sizeof(int64_t) * (size_t)(NE > 0 ? NE : 1));
    return g;
}

csrGraph* CreateEmptyUndirectedCSR(int64_t NV, int64_t NE) { return empty_csr(NV, NE * 2); }
csrGraph* CreateEmptyDirectedCSR(int64_t NV, int64_t NE) { return empty_csr(NV, NE); }

void FreeCSR(csrGraph* graph)
{
    if (!graph) return;
    free(graph->vertexPointerArray);
    free(graph->edgeArray);
    free(graph);
}

void PickRoots(int64_t* rootArrayForApproximation, int64_t NK, int64_t NV)
{
    if (NK == NV) {
        for (int64_t r = 0; r < NK; ++r) rootArrayForApproximation[r] = r;
        return;
    }
    if (NK > NV) {
        fail(SBC_ERR_ARG, "PickRoots: number of roots is greater than number of vertices");
        return;
    }
    std::vector<char> flag(NV, 0);
    for (int64_t r = 0; r < NK; ++r) {
        int64_t v = rand() % NV;
        if (flag[v]) {
            --r;
            continue;
        }
        rootArrayForApproximation[r] = v;
        flag[v] = 1;
    }
}

}  // extern "C"
