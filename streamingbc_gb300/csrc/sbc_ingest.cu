// Ingestion: DIMACS graph files parsed on all host cores, and the device-side
// part of building the slack CSR (adjacency scatter and per-vertex sort) that
// sbc_graph_create runs.
//
// ParseDimacsGraph (src/sbcMain_utils.c:382-422) reads the header line
// "NV NE" and then line u (u = 1, 2, ...) as vertex u's neighbour list: the
// leading integers of the line, ids used as they stand (1-based), reading
// stopping at the first token that is not an integer.  The graph gets NV + 1
// vertices (vertex 0, the unused 0-based slot, stays isolated) and NE is
// reported doubled (one entry per direction).  The same reading is done here
// in two passes over the file's bytes split at line boundaries, one thread per
// part: count lines and integers per line, then place the integers at their
// prefix-summed offsets.  Differences: a line is never split (the reference's
// fgets splits lines longer than 10^6 bytes and so shifts every later vertex);
// more lines than NV or an id outside 0..NV is an error (the reference writes
// past its arrays); missing trailing lines are empty neighbour lists (the
// reference leaves their offsets unset).
//
// Building the device adjacency moves the per-vertex copy and sort off the
// host: the caller's CSR is uploaded as is, a warp per vertex scatters its
// neighbours into the slack layout as int32, and each list is sorted on the
// device (a warp bitonic network in registers for up to 32 neighbours; a
// block bitonic network in shared memory, or in global scratch beyond 8192,
// for longer lists, skipped when a list is already sorted).
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "sbc_gb300.h"
#include "sbc_host.h"
#include "streamingbc.h"

namespace sbc {

// col[row[v] + i] = adj[off[v] + i] for the listed vertices' live neighbours.
__global__ void k_scatter_adjacency(int64_t nv, const int64_t* __restrict__ off, const int64_t* __restrict__ adj,
                                    const int64_t* __restrict__ row, int32_t* __restrict__ col)
{
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t v = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < nv; v += nw) {
        const int64_t b = off[v], d = off[v + 1] - b, r = row[v];
        for (int64_t i = lane; i < d; i += 32) col[r + i] = (int32_t)adj[b + i];
    }
}

// Warp per listed vertex of at most 32 neighbours: bitonic sort in registers.
__global__ void k_sort_short(const int32_t* __restrict__ list, int n, const int64_t* __restrict__ row,
                             const int32_t* __restrict__ deg, int32_t* __restrict__ col)
{
    const int lane = threadIdx.x & 31;
    const int nw = (int)(((int64_t)gridDim.x * blockDim.x) >> 5);
    for (int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n; i += nw) {
        const int v = list[i];
        const int d = deg[v];
        int32_t* c = col + row[v];
        int x = lane < d ? c[lane] : INT_MAX;
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                const int y = __shfl_xor_sync(0xffffffffu, x, j);
                const bool up = (lane & k) == 0;
                const bool low = (lane & j) == 0;
                x = (low == up) ? min(x, y) : max(x, y);
            }
        }
        if (lane < d) c[lane] = x;
    }
}

constexpr int kSortNT = 512;
constexpr int kSortShared = 8192;  // ints of a block's shared sort buffer

// Block per listed vertex of more than 32 neighbours: bitonic sort over the
// list padded to a power of two, in shared memory up to kSortShared entries
// and otherwise in the global scratch at tmp + tmp_off[i].  Lists already in
// order are left alone.
__global__ void __launch_bounds__(kSortNT) k_sort_long(const int32_t* __restrict__ list, int n,
                                                       const int64_t* __restrict__ row, const int32_t* __restrict__ deg,
                                                       int32_t* __restrict__ col, int32_t* __restrict__ tmp,
                                                       const int64_t* __restrict__ tmp_off)
{
    __shared__ int32_t s_buf[kSortShared];
    __shared__ int s_unsorted;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const int v = list[i];
        const int d = deg[v];
        int32_t* c = col + row[v];
        if (threadIdx.x == 0) s_unsorted = 0;
        __syncthreads();
        int bad = 0;
        for (int t = threadIdx.x; t + 1 < d; t += kSortNT) bad |= c[t] > c[t + 1];
        if (bad) s_unsorted = 1;
        __syncthreads();
        const int unsorted = s_unsorted;
        __syncthreads();  // every thread has read the flag before it is reset
        if (!unsorted) continue;
        int pad = 1;
        while (pad < d) pad <<= 1;
        int32_t* s = pad <= kSortShared ? s_buf : tmp + tmp_off[i];
        for (int t = threadIdx.x; t < pad; t += kSortNT) s[t] = t < d ? c[t] : INT_MAX;
        __syncthreads();
        for (int k = 2; k <= pad; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = threadIdx.x; t < pad; t += kSortNT) {
                    const int u = t ^ j;
                    if (u > t) {
                        const int32_t a = s[t], b = s[u];
                        if ((a > b) == ((t & k) == 0)) {
                            s[t] = b;
                            s[u] = a;
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int t = threadIdx.x; t < d; t += kSortNT) c[t] = s[t];
        __syncthreads();
    }
}

// Device part of building a graph's slack CSR from the caller's host CSR:
// the slack layout (row, deg) is already on the device; col receives every
// vertex's neighbours, each list sorted.  Synchronous on stream s.
cudaError_t build_adjacency(int64_t nv, const int64_t* off, const int64_t* adj, const int64_t* d_row,
                            const int32_t* d_deg, const std::vector<int32_t>& deg, int32_t* d_col, int sm_count,
                            cudaStream_t s)
{
    const int64_t ne = off[nv];
    cudaError_t e;
    int64_t *d_off = nullptr, *d_adj = nullptr, *d_tmp_off = nullptr;
    int32_t *d_short = nullptr, *d_long = nullptr, *d_tmp = nullptr;
    std::vector<int32_t> shortl, longl;
    std::vector<int64_t> tmp_off;
    int64_t tmp_total = 0;
    for (int64_t v = 0; v < nv; ++v) {
        if (deg[v] <= 1) continue;
        if (deg[v] > (1 << 30)) return cudaErrorInvalidValue;  // the sort pads lists to a power of two in int
        if (deg[v] <= 32) {
            shortl.push_back((int32_t)v);
        } else {
            longl.push_back((int32_t)v);
            int64_t pad = 1;
            while (pad < deg[v]) pad <<= 1;
            tmp_off.push_back(tmp_total);
            if (pad > kSortShared) tmp_total += pad;
        }
    }
    auto cleanup = [&]() {
        for (void* p : {(void*)d_off, (void*)d_adj, (void*)d_tmp_off, (void*)d_short, (void*)d_long, (void*)d_tmp})
            if (p) cudaFree(p);
    };
    if ((e = cudaMalloc(&d_off, sizeof(int64_t) * (nv + 1))) ||
        (e = cudaMalloc(&d_adj, sizeof(int64_t) * std::max<int64_t>(ne, 1))) ||
        (e = cudaMalloc(&d_short, sizeof(int32_t) * std::max<size_t>(shortl.size(), 1))) ||
        (e = cudaMalloc(&d_long, sizeof(int32_t) * std::max<size_t>(longl.size(), 1))) ||
        (e = cudaMalloc(&d_tmp_off, sizeof(int64_t) * std::max<size_t>(tmp_off.size(), 1))) ||
        (e = cudaMalloc(&d_tmp, sizeof(int32_t) * std::max<int64_t>(tmp_total, 1))) ||
        (e = cudaMemcpyAsync(d_off, off, sizeof(int64_t) * (nv + 1), cudaMemcpyHostToDevice, s)) ||
        (ne && (e = cudaMemcpyAsync(d_adj, adj, sizeof(int64_t) * ne, cudaMemcpyHostToDevice, s))) ||
        (!shortl.empty() &&
         (e = cudaMemcpyAsync(d_short, shortl.data(), sizeof(int32_t) * shortl.size(), cudaMemcpyHostToDevice, s))) ||
        (!longl.empty() &&
         ((e = cudaMemcpyAsync(d_long, longl.data(), sizeof(int32_t) * longl.size(), cudaMemcpyHostToDevice, s)) ||
          (e = cudaMemcpyAsync(d_tmp_off, tmp_off.data(), sizeof(int64_t) * tmp_off.size(), cudaMemcpyHostToDevice,
                               s))))) {
        cleanup();
        return e;
    }
    const int grid = sm_count * 8;
    if (nv) k_scatter_adjacency<<<grid, 256, 0, s>>>(nv, d_off, d_adj, d_row, d_col);
    if (!shortl.empty()) k_sort_short<<<grid, 256, 0, s>>>(d_short, (int)shortl.size(), d_row, d_deg, d_col);
    if (!longl.empty())
        k_sort_long<<<(int)std::min<size_t>(longl.size(), (size_t)sm_count * 4), kSortNT, 0, s>>>(
            d_long, (int)longl.size(), d_row, d_deg, d_col, d_tmp, d_tmp_off);
    if ((e = cudaGetLastError()) || (e = cudaStreamSynchronize(s))) {
        cleanup();
        return e;
    }
    cleanup();
    return cudaSuccess;
}

}  // namespace sbc

namespace {

struct Part {
    size_t b = 0, e = 0;
    std::vector<int32_t> cnt;  // integers read on each line of the part
};

inline bool space(char ch) { return ch == ' ' || ch == '\t' || ch == '\r' || ch == '\v' || ch == '\f'; }

// Reads the leading integers of the line starting at p (up to the newline or
// end); calls put(value) for each and returns the position after the line.
template <class Put>
size_t read_line(const char* buf, size_t p, size_t end, Put put)
{
    bool stopped = false;
    while (p < end && buf[p] != '\n') {
        if (space(buf[p])) {
            ++p;
            continue;
        }
        if (!stopped) {
            size_t q = p;
            bool neg = false;
            if (buf[q] == '-' || buf[q] == '+') neg = buf[q++] == '-';
            if (q < end && buf[q] >= '0' && buf[q] <= '9') {
                long long x = 0;
                while (q < end && buf[q] >= '0' && buf[q] <= '9') {
                    if (x < (LLONG_MAX - 9) / 10) x = x * 10 + (buf[q] - '0');
                    ++q;
                }
                put(neg ? -x : x);
                p = q;
                continue;
            }
            stopped = true;  // the first token that is not an integer ends the list
        }
        ++p;
    }
    return p < end ? p + 1 : p;
}

// The reading described at the top; *header_ne is the header's NE.
int dimacs_read(const char* path, int64_t* nv_out, int64_t* ne_out, int64_t** off_out, int64_t** adj_out,
                int64_t* header_ne)
{
    if (!path || !nv_out || !off_out || !adj_out) return sbc::report_error(SBC_ERR_ARG, "sbc_dimacs_read: null");
    *off_out = *adj_out = nullptr;
    FILE* fp = fopen(path, "rb");
    if (!fp) return sbc::report_error(SBC_ERR_ARG, "sbc_dimacs_read: cannot open %s", path);
    std::vector<char> buf;
    {
        char chunk[1 << 16];
        size_t k;
        while ((k = fread(chunk, 1, sizeof chunk, fp)) > 0) buf.insert(buf.end(), chunk, chunk + k);
        fclose(fp);
    }
    const size_t size = buf.size();
    // header: "NV NE ..."
    std::vector<long long> head;
    const size_t body = read_line(buf.data(), 0, size, [&](long long x) { head.push_back(x); });
    if (head.size() < 2 || head[0] < 0 || head[0] >= INT32_MAX - 1 || head[1] < 0)
        return sbc::report_error(SBC_ERR_ARG, "sbc_dimacs_read: %s has no \"NV NE\" header", path);
    const int64_t NV = head[0];
    // parts at line boundaries
    unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
    if (size - body < ((size_t)1 << 20)) nt = 1;
    std::vector<Part> parts(nt);
    for (unsigned t = 0; t < nt; ++t) {
        size_t b = body + (size - body) * t / nt;
        if (t > 0) {
            while (b < size && buf[b - 1] != '\n') ++b;
        }
        parts[t].b = b;
    }
    for (unsigned t = 0; t < nt; ++t) parts[t].e = t + 1 < nt ? parts[t + 1].b : size;
    auto run = [&](auto fn) {
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nt; ++t) th.emplace_back(fn, t);
        fn(0u);
        for (auto& x : th) x.join();
    };
    run([&](unsigned t) {
        Part& P = parts[t];
        for (size_t p = P.b; p < P.e;) {
            int32_t c = 0;
            p = read_line(buf.data(), p, P.e, [&](long long) { ++c; });
            P.cnt.push_back(c);
        }
    });
    int64_t lines = 0, ne = 0;
    for (auto& P : parts) lines += (int64_t)P.cnt.size();
    if (lines > NV) return sbc::report_error(SBC_ERR_ARG, "sbc_dimacs_read: %s has %lld adjacency lines for %lld vertices",
                                             path, (long long)lines, (long long)NV);
    const int64_t nv = NV + 1;
    int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (nv + 1));
    if (!off) return sbc::report_error(SBC_ERR_NOMEM, "sbc_dimacs_read: offsets");
    off[0] = off[1] = 0;
    {
        int64_t u = 1;
        for (auto& P : parts)
            for (int32_t c : P.cnt) {
                off[u + 1] = off[u] + c;
                ++u;
            }
        for (; u < nv; ++u) off[u + 1] = off[u];
        ne = off[nv];
    }
    int64_t* adj = (int64_t*)malloc(sizeof(int64_t) * std::max<int64_t>(ne, 1));
    if (!adj) {
        free(off);
        return sbc::report_error(SBC_ERR_NOMEM, "sbc_dimacs_read: %lld neighbour entries", (long long)ne);
    }
    std::vector<int64_t> first_line(nt, 1);
    for (unsigned t = 1; t < nt; ++t) first_line[t] = first_line[t - 1] + (int64_t)parts[t - 1].cnt.size();
    std::vector<char> bad(nt, 0);
    run([&](unsigned t) {
        const Part& P = parts[t];
        int64_t u = first_line[t];
        for (size_t p = P.b; p < P.e; ++u) {
            int64_t w = off[u];
            p = read_line(buf.data(), p, P.e, [&](long long x) {
                if (x < 0 || x > NV) bad[t] = 1;
                adj[w++] = x;
            });
        }
    });
    if (std::find(bad.begin(), bad.end(), 1) != bad.end()) {
        free(off);
        free(adj);
        return sbc::report_error(SBC_ERR_ARG, "sbc_dimacs_read: %s has a neighbour id outside 0..%lld", path,
                                 (long long)NV);
    }
    *nv_out = nv;
    if (ne_out) *ne_out = ne;
    if (header_ne) *header_ne = head[1];
    *off_out = off;
    *adj_out = adj;
    return SBC_OK;
}

}  // namespace

extern "C" {

int sbc_dimacs_read(const char* path, int64_t* nv, int64_t* ne, int64_t** off, int64_t** adj)
{
    return dimacs_read(path, nv, ne, off, adj, nullptr);
}

void sbc_free(void* p) { free(p); }

int sbc_graph_create_dimacs(sbc_graph** out, const char* path, int64_t* nv, int64_t* ne)
{
    if (!out) return sbc::report_error(SBC_ERR_ARG, "sbc_graph_create_dimacs: null");
    *out = nullptr;
    int64_t n = 0, m = 0, *off = nullptr, *adj = nullptr;
    int rc = sbc_dimacs_read(path, &n, &m, &off, &adj);
    if (!rc) rc = sbc_graph_create(out, n, off, adj);
    free(off);
    free(adj);
    if (!rc) {
        if (nv) *nv = n;
        if (ne) *ne = m;
    }
    return rc;
}

// src/sbcMain_utils.c:382-422: the graph through the STINGER shim, NV with
// the unused vertex 0 counted, NE doubled as the reference reports it (from
// the header); on failure *stingerGraph is NULL (sbc_last_error() says why).
void ParseDimacsGraph(char initial_graph_name[1024], struct stinger** stingerGraph, int64_t* NV, int64_t* NE)
{
    if (!stingerGraph) return;
    *stingerGraph = nullptr;
    int64_t n = 0, m = 0, he = 0, *off = nullptr, *adj = nullptr;
    if (dimacs_read(initial_graph_name, &n, &m, &off, &adj, &he)) return;
    csrGraph csr;
    csr.NV = n;
    csr.NE = m;
    csr.vertexPointerArray = off;
    csr.edgeArray = adj;
    CreateStingerFromCSR(&csr, stingerGraph);
    if (NV) *NV = n;
    if (NE) *NE = 2 * he;
    free(off);
    free(adj);
}

}  // extern "C"
