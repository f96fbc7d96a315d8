// Serving loop: many graphs resident on one GPU, insertion requests batched
// per graph as they arrive.
//
// The reference has no server; its callers apply one insertion at a time
// (stinger_insert_edge x2 + insertEdgeStreamingBC, src/sbcMain_utils.c:458-471,
// src/streamingbc.c:56-77).  Here:
//   admission   graphs are registered with their CSR and roots and admitted in
//               registration order while the sum of their device footprints
//               (adjacency + per-root state + worker scratch, estimated before
//               allocation) stays within the HBM budget; a released graph frees
//               its share once its queue is empty, and waiting graphs follow.
//               Requests for a graph not yet admitted wait in its queue.
//   batching    one scheduler thread; whenever a graph has queued requests and
//               no batch in flight, everything queued (up to max_batch) becomes
//               its next batch, launched asynchronously on the graph's own
//               stream (sbc_insert_batch_async).  Graphs run concurrently; a
//               request that arrives while its graph's batch is on the GPU joins
//               the graph's next batch (continuous batching).
//   completion  a host callback queued behind each batch stamps its completion
//               time; latency is completion minus the request's arrival time.
//   tuning      optionally (sbc_server_set_tuning) a graph registered without
//               a launch shape has its first batch applied through the
//               launch-shape autotuner, and a graph's cost model is trained on
//               the per-job costs logged over its first N insertions, after
//               which its batches are scheduled by the model.
//   eviction    an evicted graph's forest is checkpointed into host memory and
//               its device memory freed; it rejoins the admission queue and,
//               once it fits, is restored from the checkpoint (no static init)
//               with the requests that queued meanwhile.
// Per-graph order is preserved and results do not depend on how requests are
// grouped into batches, so each graph ends exactly where applying its stream
// alone ends.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "sbc_gb300.h"
#include "sbc_host.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t u, v;
    double t_arrival;  // seconds since the server's epoch
};

enum GraphState { WAITING = 0, ADMITTED = 1, RELEASED = 2, EVICTED = 3 };

struct ServerGraph {
    int id = 0;
    int64_t nv = 0, nk = 0;
    std::vector<int64_t> off, adj, roots;
    int variant = -1;
    bool auto_variant = false;  // registered without a launch shape
    bool tuned = false;         // first batch went through the autotuner
    int model_phase = 0;        // 0 not started, 1 logging costs, 2 trained (model schedule)
    int64_t logged = 0;         // insertions applied while logging
    int64_t footprint = 0;
    GraphState state = WAITING;
    bool release_requested = false;
    bool evict_requested = false;
    sbc_checkpoint* ckpt = nullptr;  // host copy of an evicted graph's forest
    sbc_graph* g = nullptr;
    sbc_forest* f = nullptr;
    std::deque<Req> pending;
    bool ready = false;       // static init finished (set by a stream callback)
    bool inflight = false;
    bool done = false;        // set by the completion callback
    double t_done = 0.0;
    std::vector<Req> batch;   // requests of the batch in flight
    int64_t submitted = 0, completed = 0, batches = 0, evictions = 0;
};

}  // namespace

struct sbc_server {
    int device = 0;
    int64_t budget = 0, used = 0;
    int max_batch = 1;
    int max_inflight = 0;  // batches on the device at once over all graphs (0 = no limit)
    bool autotune = false;     // first batch of a graph without a launch shape through the tuner
    int64_t train_n = 0;       // insertions of cost logging before a graph's model is trained (0 = off)
    int rr = 0;            // round-robin start of the launch scan
    Clock::time_point epoch;
    std::vector<std::unique_ptr<ServerGraph>> graphs;
    std::deque<int> waiting;
    std::mutex mu;
    std::condition_variable cv;       // work for the scheduler
    std::condition_variable cv_idle;  // drain waiters
    std::thread sched;
    bool stop = false;
    std::string error;  // first error met by the scheduler
    std::vector<double> lat_us;
    double t_first = -1.0, t_last = 0.0;
    int64_t completed = 0, batches = 0, submitted = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - epoch).count(); }
};

namespace {

// Device bytes a graph will hold once admitted: slack CSR (row, deg, deg0,
// nsort, cap, col, seq), per-root state (dist, dist8, dist2, level-2 masks,
// sigma, delta), BC,
// level histograms and the update workers' scratch for its launch shape.
int64_t footprint(int64_t nv, int64_t slots, int64_t nk, int variant, int sm_count)
{
    const int64_t slack = slots + std::max<int64_t>(nv * 4, slots / 8);
    const int64_t graph = (nv + 1) * 8 + nv * 16 + slack * 8;
    const int64_t state = nk * nv * 25 + nk * sbc::d2_words(nv) * 4 + nv * 8 + nk * (int64_t)sbc::kHistLevels * 4;
    int per_sm = std::max(1, sbc::update_workers_per_sm(variant));
    const int64_t workers = std::min<int64_t>((int64_t)per_sm * sm_count, nk);
    return graph + state + workers * (int64_t)WorkerScratch::per_worker(nv);
}

// The tuner times the first batch of at least this many requests (or of any
// size when batches are capped below it): a shape tuned on a handful of
// insertions would say little about full batches.
constexpr int64_t kTuneMinBatch = 64;

int default_variant(int64_t nv) { return nv <= 8192 ? 3 : (nv <= 262144 ? 5 : sbc::update_default_variant()); }

struct DoneArg {
    sbc_server* s;
    ServerGraph* sg;
};

void CUDART_CB on_batch_done(void* p)
{
    DoneArg* a = static_cast<DoneArg*>(p);
    {
        std::lock_guard<std::mutex> lk(a->s->mu);
        a->sg->done = true;
        a->sg->t_done = a->s->now();
    }
    a->s->cv.notify_all();
    a->s->cv_idle.notify_all();
    delete a;
}

void CUDART_CB on_ready(void* p)
{
    DoneArg* a = static_cast<DoneArg*>(p);
    {
        std::lock_guard<std::mutex> lk(a->s->mu);
        a->sg->ready = true;
    }
    a->s->cv.notify_all();
    a->s->cv_idle.notify_all();  // readiness is not scheduler work; drain waiters re-check
    delete a;
}

// Creates the graph and forest and queues the static init (asynchronous on
// the graph's stream; the graph's first batch queues behind it, and a stream
// callback marks the graph ready when the init is done).
int admit(sbc_server* s, ServerGraph* sg)
{
    int rc = sbc_set_device(s->device);
    if (sg->ckpt) {
        // an evicted graph: restored where it stood
        if (!rc) rc = sbc_checkpoint_restore(sg->ckpt, sg->variant, &sg->g, &sg->f);
        if (!rc) {
            sbc_checkpoint_free(sg->ckpt);
            sg->ckpt = nullptr;
        }
    } else {
        if (!rc) rc = sbc_graph_create(&sg->g, sg->nv, sg->off.data(), sg->adj.data());
        if (!rc) rc = sbc_forest_create_ex(&sg->f, sg->g, sg->nk, sg->roots.data(), 0, sg->variant);
        if (!rc) rc = sbc_static_init(sg->f);
    }
    if (!rc && cudaLaunchHostFunc(sg->g->stream, on_ready, new DoneArg{s, sg})) rc = SBC_ERR_CUDA;
    return rc;
}

void release_device(ServerGraph* sg)
{
    if (sg->f) sbc_forest_destroy(sg->f);
    if (sg->g) sbc_graph_destroy(sg->g);
    sg->f = nullptr;
    sg->g = nullptr;
}

// Something for the scheduler to do now: a finished batch to account, a
// batch to launch, a release to carry out or a waiting graph that fits.
bool pending_work(sbc_server* s)
{
    int inflight = 0;
    for (auto& p : s->graphs) inflight += p->inflight ? 1 : 0;
    const bool can_launch = s->max_inflight <= 0 || inflight < s->max_inflight;
    for (auto& p : s->graphs) {
        ServerGraph* sg = p.get();
        if (sg->inflight && sg->done) return true;
        if (can_launch && sg->state == ADMITTED && !sg->inflight && !sg->pending.empty()) return true;
        if (sg->state == ADMITTED && sg->release_requested && !sg->inflight && sg->pending.empty()) return true;
        if (sg->state == ADMITTED && sg->evict_requested && !sg->inflight && sg->ready) return true;
    }
    return !s->waiting.empty() &&
           s->used + s->graphs[s->waiting.front()]->footprint <= s->budget;
}

bool has_work(sbc_server* s) { return s->stop || pending_work(s); }

// Nothing in flight and nothing the scheduler could start: requests of graphs
// still waiting for admission (that do not fit yet) stay queued.
bool idle(sbc_server* s)
{
    for (auto& p : s->graphs)
        if (p->inflight || (p->state == ADMITTED && !p->ready)) return false;
    return !pending_work(s);
}

void scheduler(sbc_server* s)
{
    sbc_set_device(s->device);
    for (;;) {
        std::vector<ServerGraph*> launch, admit_list, free_list, evict_list;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return has_work(s); });
            bool any_inflight = false;
            for (auto& p : s->graphs) {
                ServerGraph* sg = p.get();
                if (sg->inflight && sg->done) {
                    for (const Req& r : sg->batch) s->lat_us.push_back((sg->t_done - r.t_arrival) * 1e6);
                    sg->completed += (int64_t)sg->batch.size();
                    s->completed += (int64_t)sg->batch.size();
                    s->t_last = std::max(s->t_last, sg->t_done);
                    sg->batch.clear();
                    sg->inflight = false;
                    sg->done = false;
                }
                any_inflight |= sg->inflight;
            }
            if (s->stop && !any_inflight) break;
            for (auto& p : s->graphs) {
                ServerGraph* sg = p.get();
                if (sg->state == ADMITTED && sg->release_requested && !sg->inflight && sg->pending.empty()) {
                    sg->state = RELEASED;
                    s->used -= sg->footprint;
                    free_list.push_back(sg);
                } else if (sg->state == ADMITTED && sg->evict_requested && !sg->inflight && sg->ready) {
                    // checkpointed below, before any admission of this round
                    sg->state = EVICTED;
                    sg->evict_requested = false;
                    sg->ready = false;
                    s->used -= sg->footprint;
                    s->waiting.push_back(sg->id);
                    evict_list.push_back(sg);
                }
            }
            while (!s->waiting.empty() && s->used + s->graphs[s->waiting.front()]->footprint <= s->budget) {
                ServerGraph* sg = s->graphs[s->waiting.front()].get();
                s->waiting.pop_front();
                s->used += sg->footprint;
                sg->state = ADMITTED;
                admit_list.push_back(sg);
            }
            int inflight = 0;
            for (auto& p : s->graphs) inflight += p->inflight ? 1 : 0;
            const int ng = (int)s->graphs.size();
            for (int k = 0; k < ng; ++k) {
                ServerGraph* sg = s->graphs[(s->rr + k) % ng].get();
                if (sg->state != ADMITTED || sg->inflight || sg->pending.empty()) continue;
                if (std::find(admit_list.begin(), admit_list.end(), sg) != admit_list.end()) continue;
                if (s->max_inflight > 0 && inflight >= s->max_inflight) break;
                inflight++;
                s->rr = (int)((sg->id + 1) % ng);
                const size_t take = std::min<size_t>(sg->pending.size(), (size_t)s->max_batch);
                sg->batch.assign(sg->pending.begin(), sg->pending.begin() + take);
                sg->pending.erase(sg->pending.begin(), sg->pending.begin() + take);
                sg->inflight = true;
                sg->batches++;
                s->batches++;
                launch.push_back(sg);
            }
            if (idle(s)) s->cv_idle.notify_all();
        }
        // CUDA work outside the lock (completion callbacks take the lock)
        for (ServerGraph* sg : free_list) release_device(sg);
        for (ServerGraph* sg : evict_list) {
            sbc_checkpoint* ck = nullptr;
            const int rc = sbc_checkpoint_take(sg->f, &ck);
            if (rc) {
                // the graph stays resident (and counted) if its state cannot be saved
                bool released = false;
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    if (s->error.empty()) s->error = std::string("eviction: ") + sbc_last_error();
                    released = sg->state == RELEASED;  // released meanwhile: out of the queue, not counted
                    if (!released) {
                        auto it = std::find(admit_list.begin(), admit_list.end(), sg);
                        if (it != admit_list.end()) {
                            admit_list.erase(it);  // re-admitted this round: already counted and dequeued
                        } else {
                            s->waiting.erase(std::remove(s->waiting.begin(), s->waiting.end(), sg->id),
                                             s->waiting.end());
                            s->used += sg->footprint;
                        }
                        sg->state = ADMITTED;
                        sg->ready = true;
                    }
                }
                if (released) release_device(sg);
                continue;
            }
            int64_t ne = 0, nk = 0;
            sbc_checkpoint_info(ck, nullptr, &nk, &ne, nullptr);
            release_device(sg);
            int sm_count = 0;
            cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, s->device);
            std::lock_guard<std::mutex> lk(s->mu);
            if (sg->state == RELEASED) {  // released while its checkpoint was being taken
                sbc_checkpoint_free(ck);
                continue;
            }
            sg->ckpt = ck;  // published under the lock: readers and release see it whole
            const int64_t fp = footprint(sg->nv, ne, nk, sg->variant, sm_count);  // the graph has grown
            if (sg->state == ADMITTED) s->used += fp - sg->footprint;  // re-admitted in this round
            sg->footprint = fp;
            sg->evictions++;
        }
        for (ServerGraph* sg : admit_list) {
            int rc = admit(s, sg);
            if (rc) {
                std::lock_guard<std::mutex> lk(s->mu);
                if (s->error.empty()) s->error = std::string("admission: ") + sbc_last_error();
                sg->ready = true;
            }
        }
        if (!admit_list.empty()) s->cv.notify_all();  // their queued requests can launch now
        for (ServerGraph* sg : launch) {
            std::vector<int64_t> u(sg->batch.size()), v(sg->batch.size());
            for (size_t i = 0; i < sg->batch.size(); ++i) {
                u[i] = sg->batch[i].u;
                v[i] = sg->batch[i].v;
            }
            const int64_t n = (int64_t)u.size();
            int rc = 0;
            if (s->autotune && sg->auto_variant && !sg->tuned && (n >= kTuneMinBatch || s->max_batch < kTuneMinBatch)) {
                // the tuner applies this batch after timing it under every shape
                sg->tuned = true;
                rc = sbc_forest_autotune(sg->f, n, u.data(), v.data(), 1, nullptr, nullptr, 0);
            } else {
                if (s->train_n > 0 && sg->model_phase == 0) {
                    rc = sbc_cost_log_start(sg->f, std::min<int64_t>(s->train_n * sg->nk, (int64_t)1 << 26));
                    sg->model_phase = 1;
                }
                if (!rc) rc = sbc_insert_batch_async(sg->f, n, u.data(), v.data());
                if (!rc && sg->model_phase == 1 && (sg->logged += n) >= s->train_n) {
                    // enough logged jobs: train (waits for this batch) and switch
                    // the graph to the model's schedule
                    int64_t samples = 0;
                    sbc_model_stats ms;
                    rc = sbc_cost_log_stop(sg->f, &samples);
                    // minibatches of up to 4096 (a multiple of 128) of the 90 %
                    // trained on; too few jobs logged: the static schedule stays
                    const int64_t ntr = samples - (int64_t)((double)samples * 0.1);
                    const int mb = (int)std::min<int64_t>(4096, ntr / 128 * 128);
                    if (!rc && mb >= 128) rc = sbc_cost_model_train(sg->f, 4, mb, 2e-3, 0.1, 1, &ms);
                    if (!rc && mb >= 128) rc = sbc_set_schedule(sg->f, SBC_SCHED_MODEL);
                    sg->model_phase = 2;
                }
            }
            cudaError_t e = cudaSuccess;
            if (!rc) e = cudaLaunchHostFunc(sg->g->stream, on_batch_done, new DoneArg{s, sg});
            if (rc || e) {
                std::lock_guard<std::mutex> lk(s->mu);
                if (s->error.empty())
                    s->error = rc ? std::string("batch: ") + sbc_last_error() : cudaGetErrorString(e);
                sg->done = true;  // count the batch as finished so the loop does not stall
                sg->t_done = s->now();
            }
        }
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->cv_idle.notify_all();
    }
}

}  // namespace

extern "C" {

int sbc_server_create(sbc_server** out, int device, int64_t hbm_budget_bytes, int max_batch)
{
    if (!out || hbm_budget_bytes <= 0 || max_batch < 1) return SBC_ERR_ARG;
    if (sbc_set_device(device)) return SBC_ERR_CUDA;
    sbc_server* s = new sbc_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_batch = max_batch;
    s->epoch = Clock::now();
    s->sched = std::thread(scheduler, s);
    *out = s;
    return SBC_OK;
}

int sbc_server_set_tuning(sbc_server* s, int autotune, int64_t train_insertions)
{
    if (!s || train_insertions < 0) return SBC_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->autotune = autotune != 0;
        s->train_n = train_insertions;
    }
    return SBC_OK;
}

int sbc_server_set_max_inflight(sbc_server* s, int max_inflight)
{
    if (!s || max_inflight < 0) return SBC_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->max_inflight = max_inflight;
    }
    s->cv.notify_all();
    return SBC_OK;
}

int sbc_server_destroy(sbc_server* s)
{
    if (!s) return SBC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    s->sched.join();
    sbc_set_device(s->device);
    for (auto& p : s->graphs) {
        if (p->g) cudaStreamSynchronize(p->g->stream);
        release_device(p.get());
        sbc_checkpoint_free(p->ckpt);
        p->ckpt = nullptr;
    }
    delete s;
    return SBC_OK;
}

int sbc_server_add_graph(sbc_server* s, int64_t nv, const int64_t* off, const int64_t* adj, int64_t nk,
                         const int64_t* roots, int variant, int* id)
{
    if (!s || nv <= 0 || !off || (!adj && off[nv] > 0) || nk <= 0 || nk > nv || !roots || !id ||
        variant >= sbc::update_variant_count())
        return SBC_ERR_ARG;
    auto sg = std::make_unique<ServerGraph>();
    sg->nv = nv;
    sg->nk = nk;
    sg->off.assign(off, off + nv + 1);
    sg->adj.assign(adj, adj + off[nv]);
    sg->roots.assign(roots, roots + nk);
    sg->variant = variant >= 0 ? variant : default_variant(nv);
    sg->auto_variant = variant < 0;
    int sm_count = 0;
    if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, s->device)) return SBC_ERR_CUDA;
    sg->footprint = footprint(nv, off[nv], nk, sg->variant, sm_count);
    std::lock_guard<std::mutex> lk(s->mu);
    if (sg->footprint > s->budget) return SBC_ERR_NOMEM;
    sg->id = (int)s->graphs.size();
    *id = sg->id;
    s->waiting.push_back(sg->id);
    s->graphs.push_back(std::move(sg));
    s->cv.notify_all();
    return SBC_OK;
}

int sbc_server_graph_info(sbc_server* s, int id, int* state, int64_t* footprint_bytes, int64_t* completed,
                          int64_t* batches)
{
    if (!s) return SBC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (id < 0 || id >= (int)s->graphs.size()) return SBC_ERR_ARG;
    ServerGraph* sg = s->graphs[id].get();
    if (state) *state = (int)sg->state;
    if (footprint_bytes) *footprint_bytes = sg->footprint;
    if (completed) *completed = sg->completed;
    if (batches) *batches = sg->batches;
    return SBC_OK;
}

static int submit_locked(sbc_server* s, int id, int64_t u, int64_t v, double t_arrival)
{
    if (id < 0 || id >= (int)s->graphs.size()) return SBC_ERR_ARG;
    ServerGraph* sg = s->graphs[id].get();
    if (sg->state == RELEASED || sg->release_requested) return SBC_ERR_STATE;
    sg->pending.push_back(Req{u, v, t_arrival});
    sg->submitted++;
    s->submitted++;
    if (s->t_first < 0.0 || t_arrival < s->t_first) s->t_first = t_arrival;
    return SBC_OK;
}

int sbc_server_submit(sbc_server* s, int id, int64_t u, int64_t v)
{
    if (!s) return SBC_ERR_ARG;
    int rc;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        rc = submit_locked(s, id, u, v, s->now());
    }
    if (!rc) s->cv.notify_all();
    return rc;
}

int sbc_server_play(sbc_server* s, int64_t n, const int32_t* graph, const int64_t* u, const int64_t* v,
                    const double* t_offset_s)
{
    if (!s || n < 0 || (n > 0 && (!graph || !u || !v || !t_offset_s))) return SBC_ERR_ARG;
    const double t0 = s->now();
    int64_t i = 0;
    while (i < n) {
        const double due = t0 + t_offset_s[i];
        double t = s->now();
        while (t < due) {
            if (due - t > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds(50));
            t = s->now();
        }
        // every request already due is submitted under one lock
        int rc = SBC_OK;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (; i < n && t0 + t_offset_s[i] <= t && !rc; ++i)
                rc = submit_locked(s, graph[i], u[i], v[i], t0 + t_offset_s[i]);
        }
        s->cv.notify_all();
        if (rc) return rc;
    }
    return SBC_OK;
}

int sbc_server_drain(sbc_server* s)
{
    if (!s) return SBC_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv.notify_all();
    // re-checked at every notification and at least every 10 ms
    while (!(idle(s) || s->stop || !s->error.empty()))
        s->cv_idle.wait_for(lk, std::chrono::milliseconds(10));
    return s->error.empty() ? SBC_OK : SBC_ERR_STATE;
}

const char* sbc_server_error(sbc_server* s)
{
    if (!s) return "";
    std::lock_guard<std::mutex> lk(s->mu);
    return s->error.c_str();
}

int sbc_server_release(sbc_server* s, int id)
{
    if (!s) return SBC_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < 0 || id >= (int)s->graphs.size()) return SBC_ERR_ARG;
        ServerGraph* sg = s->graphs[id].get();
        sg->release_requested = true;
        if (sg->state == WAITING || sg->state == EVICTED) {
            s->waiting.erase(std::remove(s->waiting.begin(), s->waiting.end(), id), s->waiting.end());
            sg->state = RELEASED;
            sg->pending.clear();
            sbc_checkpoint_free(sg->ckpt);
            sg->ckpt = nullptr;
        }
    }
    s->cv.notify_all();
    return SBC_OK;
}

int sbc_server_evict(sbc_server* s, int id)
{
    if (!s) return SBC_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < 0 || id >= (int)s->graphs.size()) return SBC_ERR_ARG;
        ServerGraph* sg = s->graphs[id].get();
        if (sg->state == RELEASED || sg->release_requested) return SBC_ERR_STATE;
        if (sg->state != ADMITTED) return SBC_OK;  // not on the device
        sg->evict_requested = true;
    }
    s->cv.notify_all();
    return SBC_OK;
}

int sbc_server_read(sbc_server* s, int id, int32_t* dist, int64_t* sigma, double* bc)
{
    if (!s) return SBC_ERR_ARG;
    ServerGraph* sg;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < 0 || id >= (int)s->graphs.size()) return SBC_ERR_ARG;
        sg = s->graphs[id].get();
        if (sg->state == EVICTED && sg->pending.empty() && sg->ckpt)
            return sbc_checkpoint_read(sg->ckpt, dist, sigma, bc);  // the host copy is the state
        if (sg->state != ADMITTED || sg->inflight || !sg->pending.empty() || !sg->f || sg->evict_requested)
            return SBC_ERR_STATE;
    }
    sbc_set_device(s->device);
    int rc = sbc_sync(sg->f);
    if (!rc && dist) rc = sbc_get_dist(sg->f, 0, sg->nk, dist);
    if (!rc && sigma) rc = sbc_get_sigma(sg->f, 0, sg->nk, sigma);
    if (!rc && bc) rc = sbc_get_bc(sg->f, bc);
    return rc;
}

int sbc_server_get_stats(sbc_server* s, sbc_server_stats* st, int reset)
{
    if (!s || !st) return SBC_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(st, 0, sizeof *st);
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->batches = s->batches;
    st->bytes_budget = s->budget;
    st->bytes_admitted = s->used;
    for (auto& p : s->graphs) {
        if (p->state == ADMITTED) st->graphs_admitted++;
        if (p->state == WAITING || p->state == EVICTED) st->graphs_waiting++;
    }
    std::vector<double> l = s->lat_us;
    if (!l.empty()) {
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) { return l[std::min(l.size() - 1, (size_t)(q * (double)(l.size() - 1) + 0.5))]; };
        st->p50_us = pct(0.50);
        st->p99_us = pct(0.99);
        st->max_us = l.back();
        double sum = 0;
        for (double x : l) sum += x;
        st->mean_us = sum / (double)l.size();
        const double span = s->t_last - s->t_first;
        st->throughput = span > 0 ? (double)l.size() / span : 0.0;
        st->mean_batch = s->batches ? (double)s->completed / (double)s->batches : 0.0;
    }
    if (reset) {
        s->lat_us.clear();
        s->completed = 0;
        s->batches = 0;
        s->submitted = 0;
        s->t_first = -1.0;
        s->t_last = 0.0;
    }
    return SBC_OK;
}

}  // extern "C"
