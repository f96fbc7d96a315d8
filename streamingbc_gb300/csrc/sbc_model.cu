// Learned per-root cost model and the batch schedule it drives.
//
// The reference orders roots for its COARSE loop by a static estimate when
// loadBalancing is BALANCE: a qsort of 2 * edgesBelow + edgesAbove per root
// (src/streamingbc.c:171-188).  Here the persistent update kernel pulls roots
// from a queue, so the order of the queue decides the tail of the launch; a
// small FP32 MLP predicts each (insertion, root) job's touched-vertex count
// from eight features available at batch start, and the roots of a batch are
// queued longest predicted batch cost first (LPT).  The model only orders
// work: results never depend on it, and the static order (classify order) is
// the fallback.  Training data are the touched-vertex counts the update kernel
// itself logs per job.
//
// Kernels (all FP32 on the CUDA cores; the MLP is 4.8k parameters, far too
// small for the tensor cores to matter):
//   k_level_hist     vertices per level of every root's tree (after static init;
//                    jobs then keep it exact as case-2 descents move vertices)
//   k_features       warp per root, lane per insertion: features of each active
//                    pair; optionally the MLP forward and the root's batch cost
//   k_order_*        counting sort of the active roots by log2 predicted cost
//                    (8 buckets per doubling), longest first, into the worklist
//   k_log_append     (features, log(1 + touched)) of the batch's jobs appended
//                    to the training set
//   k_moments        feature means / standard deviations of the training set
//   k_mlp_grad       forward + backward of 128 samples per CTA, per-CTA weight
//                    gradient sums added into one gradient buffer
//   k_adam           Adam step over the 4,801 trained parameters
//   k_mlp_eval       held-out absolute / squared error, and that of predicting
//                    the training mean
#include <cmath>
#include "sbc_host.h"
#include "sbc_internal.cuh"

namespace sbc {

// ---------------------------------------------------------------- forward

// MLP forward of one sample of raw features xr; P holds kModelParams floats.
__device__ __forceinline__ float mlp_forward(const float* __restrict__ P, const float* xr)
{
    float x[kIn];
#pragma unroll
    for (int k = 0; k < kIn; ++k) x[k] = (xr[k] - P[OFF_MU + k]) * P[OFF_ISD + k];
    float h1[kH];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
        float a = P[OFF_B1 + j];
#pragma unroll
        for (int k = 0; k < kIn; ++k) a = fmaf(P[OFF_W1 + k * kH + j], x[k], a);
        h1[j] = fmaxf(a, 0.f);
    }
    float out = P[OFF_B3];
#pragma unroll 1
    for (int j = 0; j < kH; ++j) {
        float a = P[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < kH; ++i) a = fmaf(P[OFF_W2 + i * kH + j], h1[i], a);
        out = fmaf(P[OFF_W3 + j], fmaxf(a, 0.f), out);
    }
    return out;
}

// ---------------------------------------------------------------- features

struct FeatArgs {
    const int32_t* dist;
    const uint8_t* dist8;
    const int64_t* sigma;
    const int32_t* deg0;
    const int32_t* lvlhist;
    int64_t nv;
    int nk;
    int nins;
    const int32_t* ins_u;
    const int32_t* ins_v;
    const int32_t* ins_ok;
    float* feat;          // [nk][nins][kIn] or null
    float* root_cost;     // [nk] or null
    const float* params;  // model, or null (no prediction)
};

// Features of insertion i for root r, endpoints ordered a (shallower), b:
//   d(r,a), d(r,b) (64 if unreachable), level difference (64 if b unreachable),
//   log1p deg(a), log1p deg(b), log1p |sigma(r,a)|, log1p |sigma(r,b)|,
//   log1p(vertices at level d(r,a)+1, where the descent from b starts).
// Returns false if the pair needs no job (insertion not live, or same level).
__device__ __forceinline__ bool pair_features(const FeatArgs& A, int r, int i, float f[kIn])
{
    if (A.ins_ok[i] <= 0) return false;
    const int32_t* D = A.dist + (size_t)r * A.nv;
    const int u = A.ins_u[i], v = A.ins_v[i];
    const int du = D[u], dv = D[v];
    if (du == dv) return false;
    const int a = du < dv ? u : v, b = du < dv ? v : u;
    const int da = min(du, dv), db = max(du, dv);
    const int64_t* S = A.sigma + (size_t)r * A.nv;
    const int32_t* H = A.lvlhist + (size_t)r * kHistLevels;
    f[0] = (float)min(da, 63);
    f[1] = db == SBC_INF ? 64.f : (float)min(db, 63);
    f[2] = db == SBC_INF ? 64.f : (float)min(db - da, 63);
    f[3] = log1pf((float)A.deg0[a]);
    f[4] = log1pf((float)A.deg0[b]);
    // sigma is int64 with wrap-around (as in the reference); a wrapped count
    // is negative, so its magnitude is taken to keep the feature finite
    f[5] = log1pf(fabsf((float)S[a]));
    f[6] = db == SBC_INF ? 0.f : log1pf(fabsf((float)S[b]));
    f[7] = log1pf((float)H[min(da + 1, kHistLevels - 1)]);
    return true;
}

// Warp per root, lanes over the batch's insertions.
__global__ void __launch_bounds__(256) k_features(const __grid_constant__ FeatArgs A)
{
    __shared__ float P[kModelParams];
    if (A.params)
        for (int t = threadIdx.x; t < kModelParams; t += blockDim.x) P[t] = A.params[t];
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= A.nk) return;
    float cost = 0.f;
    bool active = false;
#pragma unroll 1
    for (int i = lane; i < A.nins; i += 32) {
        float f[kIn];
        if (!pair_features(A, r, i, f)) continue;
        active = true;
        if (A.feat) {
            float* o = A.feat + ((size_t)r * A.nins + i) * kIn;
#pragma unroll
            for (int k = 0; k < kIn; ++k) o[k] = f[k];
        }
        if (A.params) cost += fmaxf(expm1f(mlp_forward(P, f)), 0.f);
    }
    active = __any_sync(full, active);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cost += __shfl_xor_sync(full, cost, o);
    if (lane == 0 && A.root_cost) A.root_cost[r] = active ? cost : -1.f;
}

// ---------------------------------------------------------------- ordering

__device__ __forceinline__ int cost_bucket(float c)
{
    const int k = (int)(log2f(c + 1.f) * 8.f);
    return kCostBuckets - 1 - min(max(k, 0), kCostBuckets - 1);  // longest first
}

__global__ void k_order_count(const float* __restrict__ root_cost, int nk, int* __restrict__ cnt)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nk && root_cost[r] >= 0.f) atomicAdd(&cnt[cost_bucket(root_cost[r])], 1);
}

// counts -> exclusive offsets (one CTA of kCostBuckets threads); nwork[0] =
// active roots, nwork[1] (the update kernel's work counter) = 0.
__global__ void __launch_bounds__(kCostBuckets) k_order_scan(int* __restrict__ cnt, int* __restrict__ nwork)
{
    __shared__ int warp[kCostBuckets / 32];
    int total;
    const int c = cnt[threadIdx.x];
    const int off = block_exclusive_scan<kCostBuckets>(c, warp, &total);
    cnt[threadIdx.x] = off;
    if (threadIdx.x == 0) {
        nwork[0] = total;
        nwork[1] = 0;
    }
}

__global__ void k_order_scatter(const float* __restrict__ root_cost, int nk, int* __restrict__ off,
                                int* __restrict__ worklist)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < nk && root_cost[r] >= 0.f) worklist[atomicAdd(&off[cost_bucket(root_cost[r])], 1)] = r;
}

// ---------------------------------------------------------------- logging

__global__ void k_log_append(const float* __restrict__ feat, const int32_t* __restrict__ cost_log, int64_t pairs,
                             float* __restrict__ x, float* __restrict__ y, unsigned long long* __restrict__ n,
                             int64_t capacity)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= pairs) return;
    const int32_t c = cost_log[p];
    if (c < 0) return;
    const unsigned long long idx = atomicAdd(n, 1ULL);
    if ((int64_t)idx >= capacity) return;
#pragma unroll
    for (int k = 0; k < kIn; ++k) x[idx * kIn + k] = feat[p * kIn + k];
    y[idx] = log1pf((float)c);
}

// Vertices per level (levels from the one-byte shadow; 254 = deep, 255 =
// unreachable) of every root's tree: CTA per root.
__global__ void k_level_hist(const uint8_t* __restrict__ dist8, int64_t nv, int32_t* __restrict__ hist,
                             const int* __restrict__ list, const int* __restrict__ nlist)
{
    __shared__ int h[kHistLevels];
    if (list && (int)blockIdx.x >= *nlist) return;
    const size_t r = list ? (size_t)list[blockIdx.x] : blockIdx.x;
    for (int t = threadIdx.x; t < kHistLevels; t += blockDim.x) h[t] = 0;
    __syncthreads();
    const uint8_t* D8 = dist8 + r * nv;
    for (int64_t v = threadIdx.x; v < nv; v += blockDim.x) {
        const int d = D8[v];
        if (d != SBC_D8_INF) atomicAdd(&h[min(d, kHistLevels - 1)], 1);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kHistLevels; t += blockDim.x) hist[r * kHistLevels + t] = h[t];
}

// ---------------------------------------------------------------- training

// Feature sums, sums of squares and the target sum over samples [0, n):
// sums[0..7] sum x, [8..15] sum x^2, [16] sum y.
__global__ void k_moments(const float* __restrict__ x, const float* __restrict__ y, int64_t n, double* sums)
{
    float s[kIn] = {}, q[kIn] = {}, sy = 0.f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
#pragma unroll
        for (int k = 0; k < kIn; ++k) {
            const float v = x[j * kIn + k];
            s[k] += v;
            q[k] = fmaf(v, v, q[k]);
        }
        sy += y[j];
    }
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < kIn; ++k) {
            s[k] += __shfl_xor_sync(full, s[k], o);
            q[k] += __shfl_xor_sync(full, q[k], o);
        }
        sy += __shfl_xor_sync(full, sy, o);
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < kIn; ++k) {
            atomicAdd(&sums[k], (double)s[k]);
            atomicAdd(&sums[kIn + k], (double)q[k]);
        }
        atomicAdd(&sums[2 * kIn], (double)sy);
    }
}

constexpr int kGradThreads = 128;
constexpr int kLd = kGradThreads + 1;  // row stride of the per-CTA activation tiles (odd: no bank conflicts)
constexpr int kParamPad = (kModelParams + 3) & ~3;
constexpr size_t kGradSmem = sizeof(float) * ((size_t)kParamPad + (size_t)kIn * kLd + 4 * (size_t)kH * kLd + kLd);

struct GradArgs {
    const float* params;
    float* grad;  // [kTrainParams], accumulated
    const float* x;
    const float* y;
    int64_t base, count;           // positions [base, base+count) of the permuted order
    int64_t mul, add, mod;         // position j -> sample (j * mul + add) % mod
    float scale;                   // d loss / d out = scale * (out - y): 2 / minibatch size
    float* pred_out;               // [count] predictions, or null
};

// Forward and backward of the mean squared error for kGradThreads samples
// (thread per sample); the CTA's weight-gradient sums are added into grad.
__global__ void __launch_bounds__(kGradThreads) k_mlp_grad(const __grid_constant__ GradArgs A)
{
    extern __shared__ float smem[];
    float* P = smem;
    float* X = P + kParamPad;     // [kIn][kLd] normalised inputs
    float* H1 = X + kIn * kLd;    // [kH][kLd] layer-1 activations
    float* H2 = H1 + kH * kLd;    // [kH][kLd] layer-2 activations
    float* D2 = H2 + kH * kLd;    // [kH][kLd] layer-2 pre-activation gradients
    float* D1 = D2 + kH * kLd;    // [kH][kLd] layer-1 pre-activation gradients
    float* Do = D1 + kH * kLd;    // [kLd] output gradients
    const int t = threadIdx.x;
    for (int i = t; i < kModelParams; i += kGradThreads) P[i] = A.params[i];
    __syncthreads();
    const int64_t j = A.base + (int64_t)blockIdx.x * kGradThreads + t;
    const bool valid = j < A.base + A.count;
    float x[kIn];
    float yv = 0.f;
    if (valid) {
        const int64_t sid = (int64_t)(((unsigned long long)j * (unsigned long long)A.mul + (unsigned long long)A.add) %
                                      (unsigned long long)A.mod);
#pragma unroll
        for (int k = 0; k < kIn; ++k) x[k] = (A.x[sid * kIn + k] - P[OFF_MU + k]) * P[OFF_ISD + k];
        yv = A.y[sid];
    } else {
#pragma unroll
        for (int k = 0; k < kIn; ++k) x[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < kIn; ++k) X[k * kLd + t] = x[k];
    float h1[kH];
#pragma unroll
    for (int jj = 0; jj < kH; ++jj) {
        float a = P[OFF_B1 + jj];
#pragma unroll
        for (int k = 0; k < kIn; ++k) a = fmaf(P[OFF_W1 + k * kH + jj], x[k], a);
        h1[jj] = fmaxf(a, 0.f);
        H1[jj * kLd + t] = h1[jj];
    }
    float out = P[OFF_B3];
    for (int j2 = 0; j2 < kH; ++j2) {
        float a = P[OFF_B2 + j2];
#pragma unroll
        for (int i = 0; i < kH; ++i) a = fmaf(P[OFF_W2 + i * kH + j2], h1[i], a);
        a = fmaxf(a, 0.f);
        H2[j2 * kLd + t] = a;
        out = fmaf(P[OFF_W3 + j2], a, out);
    }
    const float dout = valid ? A.scale * (out - yv) : 0.f;
    Do[t] = dout;
    if (A.pred_out && valid) A.pred_out[j - A.base] = out;
    for (int j2 = 0; j2 < kH; ++j2) D2[j2 * kLd + t] = H2[j2 * kLd + t] > 0.f ? dout * P[OFF_W3 + j2] : 0.f;
#pragma unroll
    for (int i = 0; i < kH; ++i) {
        float d = 0.f;
        for (int j2 = 0; j2 < kH; ++j2) d = fmaf(P[OFF_W2 + i * kH + j2], D2[j2 * kLd + t], d);
        D1[i * kLd + t] = h1[i] > 0.f ? d : 0.f;
    }
    __syncthreads();
    for (int e = t; e < kH * kH; e += kGradThreads) {
        const int i = e / kH, j2 = e % kH;
        float acc = 0.f;
        for (int s = 0; s < kGradThreads; ++s) acc = fmaf(H1[i * kLd + s], D2[j2 * kLd + s], acc);
        atomicAdd(&A.grad[OFF_W2 + e], acc);
    }
    for (int e = t; e < kIn * kH; e += kGradThreads) {
        const int k = e / kH, jj = e % kH;
        float acc = 0.f;
        for (int s = 0; s < kGradThreads; ++s) acc = fmaf(X[k * kLd + s], D1[jj * kLd + s], acc);
        atomicAdd(&A.grad[OFF_W1 + e], acc);
    }
    if (t < kH) {
        float g1 = 0.f, g2 = 0.f, g3 = 0.f;
        for (int s = 0; s < kGradThreads; ++s) {
            g1 += D1[t * kLd + s];
            g2 += D2[t * kLd + s];
            g3 = fmaf(Do[s], H2[t * kLd + s], g3);
        }
        atomicAdd(&A.grad[OFF_B1 + t], g1);
        atomicAdd(&A.grad[OFF_B2 + t], g2);
        atomicAdd(&A.grad[OFF_W3 + t], g3);
    } else if (t == kH) {
        float g = 0.f;
        for (int s = 0; s < kGradThreads; ++s) g += Do[s];
        atomicAdd(&A.grad[OFF_B3], g);
    }
}

// One Adam step (bias-corrected by c1 = 1 - beta1^t, c2 = 1 - beta2^t); the
// gradient buffer is cleared for the next step.
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int n, float lr, float beta1, float beta2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    g[i] = 0.f;
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Held-out error over samples [lo, hi), thread per sample: sums[24] |err|,
// sums[25] err^2, sums[26] |y - ymean| (the error of predicting the training mean).
__global__ void __launch_bounds__(256) k_mlp_eval(const float* __restrict__ params, const float* __restrict__ x,
                                                  const float* __restrict__ y, int64_t lo, int64_t hi, float ymean,
                                                  double* sums)
{
    __shared__ float P[kModelParams];
    for (int t = threadIdx.x; t < kModelParams; t += blockDim.x) P[t] = params[t];
    __syncthreads();
    float ae = 0.f, se = 0.f, ce = 0.f;
    const int64_t j = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < hi) {
        const float e = mlp_forward(P, x + j * kIn) - y[j];
        ae = fabsf(e);
        se = e * e;
        ce = fabsf(y[j] - ymean);
    }
    const unsigned full = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ae += __shfl_xor_sync(full, ae, o);
        se += __shfl_xor_sync(full, se, o);
        ce += __shfl_xor_sync(full, ce, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&sums[24], (double)ae);
        atomicAdd(&sums[25], (double)se);
        atomicAdd(&sums[26], (double)ce);
    }
}

__global__ void __launch_bounds__(256) k_predict(const float* __restrict__ params, const float* __restrict__ x,
                                                 int64_t n, float* __restrict__ out)
{
    __shared__ float P[kModelParams];
    for (int t = threadIdx.x; t < kModelParams; t += blockDim.x) P[t] = params[t];
    __syncthreads();
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = mlp_forward(P, x + j * kIn);
}

// ---------------------------------------------------------------- launchers

cudaError_t launch_level_hist(sbc_forest* f) { return launch_level_hist_list(f, nullptr, nullptr); }

cudaError_t launch_level_hist_list(sbc_forest* f, const int* d_list, const int* d_nlist)
{
    if (!f->d_lvlhist) return cudaSuccess;
    k_level_hist<<<(int)f->nk, 256, 0, f->g->stream>>>(f->d_dist8, f->nv, f->d_lvlhist, d_list, d_nlist);
    return cudaGetLastError();
}

cudaError_t launch_schedule(sbc_forest* f, int n, bool* built_worklist)
{
    *built_worklist = false;
    CostModel* M = f->model;
    if (!M) return cudaSuccess;
    const bool predict = f->schedule == 1 && M->trained;
    if (!predict && !M->logging) return cudaSuccess;
    sbc_graph* g = f->g;
    cudaStream_t s = g->stream;
    FeatArgs A;
    A.dist = f->d_dist;
    A.dist8 = f->d_dist8;
    A.sigma = f->d_sigma;
    A.deg0 = g->d_deg0;
    A.lvlhist = f->d_lvlhist;
    A.nv = f->nv;
    A.nk = (int)f->nk;
    A.nins = n;
    A.ins_u = g->d_ins;
    A.ins_v = g->d_ins + g->ins_capacity;
    A.ins_ok = g->d_ins + 2 * g->ins_capacity;
    A.feat = M->logging ? M->d_feat : nullptr;
    A.root_cost = predict ? M->d_root_cost : nullptr;
    A.params = predict ? M->d_params : nullptr;
    cudaError_t e;
    if (M->logging && (e = cudaMemsetAsync(M->d_cost_log, 0xff, sizeof(int32_t) * (size_t)f->nk * n, s))) return e;
    k_features<<<(int)((f->nk + 7) / 8), 256, 0, s>>>(A);
    if ((e = cudaGetLastError())) return e;
    if (!predict) return cudaSuccess;
    const int blocks = (int)((f->nk + 255) / 256);
    if ((e = cudaMemsetAsync(M->d_buckets, 0, sizeof(int) * kCostBuckets, s))) return e;
    k_order_count<<<blocks, 256, 0, s>>>(M->d_root_cost, (int)f->nk, M->d_buckets);
    k_order_scan<<<1, kCostBuckets, 0, s>>>(M->d_buckets, f->d_nwork);
    k_order_scatter<<<blocks, 256, 0, s>>>(M->d_root_cost, (int)f->nk, M->d_buckets, f->d_worklist);
    *built_worklist = true;
    return cudaGetLastError();
}

cudaError_t launch_log_append(sbc_forest* f, int n)
{
    CostModel* M = f->model;
    if (!M || !M->logging) return cudaSuccess;
    const int64_t pairs = f->nk * (int64_t)n;
    k_log_append<<<(int)((pairs + 255) / 256), 256, 0, f->g->stream>>>(M->d_feat, M->d_cost_log, pairs, M->d_x,
                                                                       M->d_y, M->d_n, M->capacity);
    return cudaGetLastError();
}

cudaError_t launch_moments(sbc_forest* f, int64_t n)
{
    CostModel* M = f->model;
    cudaStream_t s = f->g->stream;
    cudaError_t e;
    if ((e = cudaMemsetAsync(M->d_sums, 0, sizeof(double) * 32, s))) return e;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 4);
    k_moments<<<(int)std::max<int64_t>(blocks, 1), 256, 0, s>>>(M->d_x, M->d_y, n, M->d_sums);
    return cudaGetLastError();
}

cudaError_t launch_grad(const float* d_params, float* d_grad, const float* d_x, const float* d_y, int64_t base,
                        int64_t count, int64_t n, int64_t mul, int64_t add, float* d_pred, cudaStream_t s)
{
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem))) return e;
    GradArgs A;
    A.params = d_params;
    A.grad = d_grad;
    A.x = d_x;
    A.y = d_y;
    A.base = base;
    A.count = count;
    A.mul = mul;
    A.add = add;
    A.mod = n;
    A.scale = 2.f / (float)count;
    A.pred_out = d_pred;
    k_mlp_grad<<<(int)((count + kGradThreads - 1) / kGradThreads), kGradThreads, kGradSmem, s>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_train_step(sbc_forest* f, int64_t base, int64_t count, int64_t n, int64_t mul, int64_t add, float lr)
{
    CostModel* M = f->model;
    cudaStream_t s = f->g->stream;
    cudaError_t e;
    if ((e = launch_grad(M->d_params, M->d_grad, M->d_x, M->d_y, base, count, n, mul, add, nullptr, s))) return e;
    M->adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)M->adam_t), c2 = 1.f - powf(b2, (float)M->adam_t);
    k_adam<<<(kTrainParams + 255) / 256, 256, 0, s>>>(M->d_params, M->d_grad, M->d_m, M->d_v, kTrainParams, lr, b1, b2,
                                                      1e-8f, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_eval(sbc_forest* f, int64_t lo, int64_t hi, float ymean)
{
    CostModel* M = f->model;
    if (hi <= lo) return cudaSuccess;
    const int64_t blocks = (hi - lo + 255) / 256;
    k_mlp_eval<<<(int)blocks, 256, 0, f->g->stream>>>(M->d_params, M->d_x, M->d_y, lo, hi, ymean, M->d_sums);
    return cudaGetLastError();
}

cudaError_t launch_predict(const float* d_params, const float* d_x, int64_t n, float* d_out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    k_predict<<<(int)((n + 255) / 256), 256, 0, s>>>(d_params, d_x, n, d_out);
    return cudaGetLastError();
}

}  // namespace sbc
