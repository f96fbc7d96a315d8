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
    int32_t* d_ins = nullptr;  // [3 * ins_capacity]: u, v, ok
    int32_t* h_ins = nullptr;  // pinned [2 * ins_capacity]
    const int32_t** d_src = nullptr;  // device slot: addresses of the caller's endpoint arrays
    int64_t repacks = 0;
    // forests bound to this graph; destroying the graph detaches them
    std::vector<sbc_forest*> forests;

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
    int64_t* d_sigma = nullptr;
    double* d_delta = nullptr;
    double* d_bc = nullptr;
    bool initialized = false;
    // persistent workers and their scratch
    int sm_count = 0;
    int variant = 0;  // launch shape of the update kernel
    int64_t workers = 0;
    int64_t workers_req = 0;  // worker count the caller asked for (0 = one per resident CTA)
    int64_t state_bytes = 0;
    int32_t* d_st = nullptr;
    int64_t* d_dp = nullptr;
    double* d_acc = nullptr;
    int32_t* d_qd = nullptr;
    int32_t* d_qa = nullptr;
    int32_t* d_qs = nullptr;
    int32_t* d_lvl = nullptr;
    uint32_t* d_bits = nullptr;
    int* d_worklist = nullptr;
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

    sbc::ScratchBase scratch() const
    {
        sbc::ScratchBase s;
        s.st = d_st;
        s.dp = d_dp;
        s.acc = d_acc;
        s.qd = d_qd;
        s.qa = d_qa;
        s.qs = d_qs;
        s.lvl = d_lvl;
        s.bits = d_bits;
        return s;
    }
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

namespace sbc {
int static_workers_per_sm();
int update_variant_count();
int update_default_variant();
int update_variant_threads(int v);
int update_workers_per_sm(int v);
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
}  // namespace sbc
