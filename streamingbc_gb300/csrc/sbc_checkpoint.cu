// Forest checkpoints: host copies of a forest's graph and per-root state, and
// forests rebuilt from them without a static init.
//
// The reference keeps nothing of the kind: its forest lives in host records
// for the life of the process, and STINGER's own save/open
// (src/stinger/stinger.c:1808, :1936) stores the graph alone.  A checkpoint
// here is what a server needs to evict a resident graph and admit it again
// later: the live adjacency as a CSR (int64 offsets, int32 neighbours), the
// roots, every root's dist (int32) / sigma (int64) / delta (fp64) row and the
// BC vector.  Restoring builds a graph from the CSR, a forest on it, uploads
// the rows, and derives the one-byte distance shadow, the level histograms
// and the rosters from dist on the device, so the restored forest continues
// exactly where the saved one stood.
//
// File layout (little-endian, as both host architectures are): a 40-byte
// header {magic "SBCCKPT1", u32 version = 1, u32 0, i64 nv, i64 nk, i64 ne},
// then off[nv+1] i64, adj[ne] i32, roots[nk] i64, bc[nv] f64, dist[nk*nv] i32,
// sigma[nk*nv] i64, delta[nk*nv] f64.
#include <cstdio>
#include <cstring>
#include <vector>

#include "sbc_gb300.h"
#include "sbc_host.h"

struct sbc_checkpoint {
    int64_t nv = 0, nk = 0;
    std::vector<int64_t> off;
    std::vector<int32_t> adj;
    std::vector<int64_t> roots;
    std::vector<double> bc;
    std::vector<int32_t> dist;
    std::vector<int64_t> sigma;
    std::vector<double> delta;

    int64_t bytes() const
    {
        return (int64_t)(off.size() * 8 + adj.size() * 4 + roots.size() * 8 + bc.size() * 8 + dist.size() * 4 +
                         sigma.size() * 8 + delta.size() * 8);
    }
};

namespace sbc {

__global__ void k_dist8_rows(const int32_t* __restrict__ dist, uint8_t* __restrict__ dist8, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dist8[i] = enc_d8(dist[i]);
}

}  // namespace sbc

namespace {

struct FileHeader {
    char magic[8];
    uint32_t version, reserved;
    int64_t nv, nk, ne;
};
static_assert(sizeof(FileHeader) == 40, "checkpoint header layout");
constexpr char kMagic[8] = {'S', 'B', 'C', 'C', 'K', 'P', 'T', '1'};

int ck(cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return SBC_OK;
    return sbc::report_error(e == cudaErrorMemoryAllocation ? SBC_ERR_NOMEM : SBC_ERR_CUDA, "%s: %s", where,
                             cudaGetErrorString(e));
}

template <class T>
bool put(FILE* fp, const std::vector<T>& v)
{
    return v.empty() || fwrite(v.data(), sizeof(T), v.size(), fp) == v.size();
}

template <class T>
bool get(FILE* fp, std::vector<T>& v, size_t n)
{
    v.resize(n);
    return n == 0 || fread(v.data(), sizeof(T), n, fp) == n;
}

}  // namespace

extern "C" {

int sbc_checkpoint_take(sbc_forest* f, sbc_checkpoint** out)
{
    if (!f || !out) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_take: null");
    *out = nullptr;
    if (!f->g) return sbc::report_error(SBC_ERR_STATE, "sbc_checkpoint_take: the forest's graph was destroyed");
    if (!f->initialized) return sbc::report_error(SBC_ERR_STATE, "sbc_checkpoint_take before sbc_static_init");
    if (cudaSetDevice(f->device) != cudaSuccess) return sbc::report_error(SBC_ERR_CUDA, "cudaSetDevice failed");
    sbc_checkpoint* c = new sbc_checkpoint();
    c->nv = f->nv;
    c->nk = f->nk;
    c->off.resize(f->nv + 1);
    int rc = sbc_graph_to_csr(f->g, c->off.data(), nullptr);  // synchronises the graph's stream
    if (!rc) {
        std::vector<int64_t> adj64(c->off[f->nv]);
        rc = sbc_graph_to_csr(f->g, c->off.data(), adj64.data());
        c->adj.assign(adj64.begin(), adj64.end());
    }
    if (rc) {
        delete c;
        return rc;
    }
    c->roots = f->h_roots;
    const size_t cells = (size_t)f->nk * (size_t)f->nv;
    try {
        c->bc.resize(f->nv);
        c->dist.resize(cells);
        c->sigma.resize(cells);
        c->delta.resize(cells);
    } catch (...) {
        delete c;
        return sbc::report_error(SBC_ERR_NOMEM, "sbc_checkpoint_take: %lld host bytes", (long long)(cells * 20));
    }
    if ((rc = ck(cudaMemcpy(c->bc.data(), f->d_bc, sizeof(double) * f->nv, cudaMemcpyDeviceToHost), "bc")) ||
        (rc = ck(cudaMemcpy(c->dist.data(), f->d_dist, sizeof(int32_t) * cells, cudaMemcpyDeviceToHost), "dist")) ||
        (rc = ck(cudaMemcpy(c->sigma.data(), f->d_sigma, sizeof(int64_t) * cells, cudaMemcpyDeviceToHost), "sigma")) ||
        (rc = ck(cudaMemcpy(c->delta.data(), f->d_delta, sizeof(double) * cells, cudaMemcpyDeviceToHost), "delta"))) {
        delete c;
        return rc;
    }
    *out = c;
    return SBC_OK;
}

int sbc_checkpoint_restore(const sbc_checkpoint* c, int variant, sbc_graph** g_out, sbc_forest** f_out)
{
    if (!c || !g_out || !f_out) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_restore: null");
    *g_out = nullptr;
    *f_out = nullptr;
    std::vector<int64_t> adj64(c->adj.begin(), c->adj.end());
    sbc_graph* g = nullptr;
    sbc_forest* f = nullptr;
    int rc = sbc_graph_create(&g, c->nv, c->off.data(), adj64.data());
    if (!rc) rc = sbc_forest_create_ex(&f, g, c->nk, c->roots.data(), 0, variant);
    if (rc) {
        sbc_graph_destroy(g);
        return rc;
    }
    const size_t cells = (size_t)c->nk * (size_t)c->nv;
    cudaStream_t s = g->stream;
    if ((rc = ck(cudaMemcpyAsync(f->d_bc, c->bc.data(), sizeof(double) * c->nv, cudaMemcpyHostToDevice, s), "bc")) ||
        (rc = ck(cudaMemcpyAsync(f->d_dist, c->dist.data(), sizeof(int32_t) * cells, cudaMemcpyHostToDevice, s),
                 "dist")) ||
        (rc = ck(cudaMemcpyAsync(f->d_sigma, c->sigma.data(), sizeof(int64_t) * cells, cudaMemcpyHostToDevice, s),
                 "sigma")) ||
        (rc = ck(cudaMemcpyAsync(f->d_delta, c->delta.data(), sizeof(double) * cells, cudaMemcpyHostToDevice, s),
                 "delta"))) {
        sbc_forest_destroy(f);
        sbc_graph_destroy(g);
        return rc;
    }
    sbc::k_dist8_rows<<<f->sm_count * 8, 256, 0, s>>>(f->d_dist, f->d_dist8, cells);
    if ((rc = ck(cudaGetLastError(), "one-byte distances")) ||
        (rc = ck(sbc::launch_dist2_rows(f, nullptr, nullptr), "two-bit distances")) ||
        (rc = ck(sbc::launch_l2mask_build_all(f), "level-2 masks")) ||
        (rc = ck(sbc::launch_level_hist(f), "level histograms")) ||
        (rc = ck(sbc::launch_roster_build(f), "rosters")) || (rc = ck(cudaStreamSynchronize(s), "restore"))) {
        sbc_forest_destroy(f);
        sbc_graph_destroy(g);
        return rc;
    }
    f->initialized = true;
    *g_out = g;
    *f_out = f;
    return SBC_OK;
}

int sbc_checkpoint_save(const sbc_checkpoint* c, const char* path)
{
    if (!c || !path) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_save: null");
    FILE* fp = fopen(path, "wb");
    if (!fp) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_save: cannot open %s", path);
    FileHeader h;
    memcpy(h.magic, kMagic, sizeof h.magic);
    h.version = 1;
    h.reserved = 0;
    h.nv = c->nv;
    h.nk = c->nk;
    h.ne = (int64_t)c->adj.size();
    const bool ok = fwrite(&h, sizeof h, 1, fp) == 1 && put(fp, c->off) && put(fp, c->adj) && put(fp, c->roots) &&
                    put(fp, c->bc) && put(fp, c->dist) && put(fp, c->sigma) && put(fp, c->delta);
    if (fclose(fp) != 0 || !ok) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_save: write to %s failed", path);
    return SBC_OK;
}

int sbc_checkpoint_load(const char* path, sbc_checkpoint** out)
{
    if (!path || !out) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_load: null");
    *out = nullptr;
    FILE* fp = fopen(path, "rb");
    if (!fp) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_load: cannot open %s", path);
    FileHeader h;
    if (fread(&h, sizeof h, 1, fp) != 1 || memcmp(h.magic, kMagic, sizeof h.magic) != 0 || h.version != 1 ||
        h.nv < 0 || h.nv >= INT32_MAX || h.nk < 0 || h.nk > h.nv || h.ne < 0) {
        fclose(fp);
        return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_load: %s is not a forest checkpoint", path);
    }
    sbc_checkpoint* c = new sbc_checkpoint();
    c->nv = h.nv;
    c->nk = h.nk;
    const size_t cells = (size_t)h.nk * (size_t)h.nv;
    bool ok = false;
    try {
        ok = get(fp, c->off, h.nv + 1) && get(fp, c->adj, h.ne) && get(fp, c->roots, h.nk) && get(fp, c->bc, h.nv) &&
             get(fp, c->dist, cells) && get(fp, c->sigma, cells) && get(fp, c->delta, cells);
    } catch (...) {
        ok = false;
    }
    fclose(fp);
    // the CSR must be consistent before anything indexes with it
    if (ok) ok = c->off[0] == 0 && c->off[h.nv] == h.ne;
    for (int64_t v = 0; ok && v < h.nv; ++v) ok = c->off[v + 1] >= c->off[v];
    for (int64_t e = 0; ok && e < h.ne; ++e) ok = c->adj[e] >= 0 && c->adj[e] < h.nv;
    for (int64_t r = 0; ok && r < h.nk; ++r) ok = c->roots[r] >= 0 && c->roots[r] < h.nv;
    if (!ok) {
        delete c;
        return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_load: %s is truncated or inconsistent", path);
    }
    *out = c;
    return SBC_OK;
}

int sbc_checkpoint_info(const sbc_checkpoint* c, int64_t* nv, int64_t* nk, int64_t* ne, int64_t* bytes)
{
    if (!c) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_info: null");
    if (nv) *nv = c->nv;
    if (nk) *nk = c->nk;
    if (ne) *ne = (int64_t)c->adj.size();
    if (bytes) *bytes = c->bytes();
    return SBC_OK;
}

int sbc_checkpoint_read(const sbc_checkpoint* c, int32_t* dist, int64_t* sigma, double* bc)
{
    if (!c) return sbc::report_error(SBC_ERR_ARG, "sbc_checkpoint_read: null");
    if (dist && !c->dist.empty()) memcpy(dist, c->dist.data(), sizeof(int32_t) * c->dist.size());
    if (sigma && !c->sigma.empty()) memcpy(sigma, c->sigma.data(), sizeof(int64_t) * c->sigma.size());
    if (bc && !c->bc.empty()) memcpy(bc, c->bc.data(), sizeof(double) * c->bc.size());
    return SBC_OK;
}

int sbc_checkpoint_free(sbc_checkpoint* c)
{
    delete c;
    return SBC_OK;
}

}  // extern "C"
