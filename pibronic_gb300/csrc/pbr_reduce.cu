// pbr_reduce.cu -- FP64 device reductions of the per-sample outputs into estimator moments.
//
// Each thread keeps shifted sums over a strided range and turns them into (count, mean, M2)
// triples; triples are merged with Chan's pairwise formula, first across the warp by shuffles,
// then across the block in shared memory, then across blocks by a single-block second pass,
// always in the same order, so results are bitwise reproducible for a given X.
#include "pbr_common.cuh"

namespace {

constexpr int kRedThreads = 256;
constexpr int64_t kPerBlock = 4096;
constexpr int kMaxBlocks = 4096;

struct Moments { double n, mean, m2; };

__device__ __forceinline__ Moments merge(const Moments& a, const Moments& b) {
    if (a.n == 0.0) return b;
    if (b.n == 0.0) return a;
    Moments r;
    r.n = a.n + b.n;
    const double d = b.mean - a.mean;
    r.mean = a.mean + d * (b.n / r.n);
    r.m2 = a.m2 + b.m2 + d * d * (a.n * b.n / r.n);
    return r;
}

__device__ __forceinline__ Moments shfl_down(const Moments& m, int off) {
    return Moments{__shfl_down_sync(0xffffffffu, m.n, off), __shfl_down_sync(0xffffffffu, m.mean, off),
                   __shfl_down_sync(0xffffffffu, m.m2, off)};
}

// block-wide merge of V moment triples; result valid in thread 0
template <int V>
__device__ void block_merge(Moments (&m)[V]) {
    __shared__ Moments sm[kRedThreads / 32][V];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const Moments o = shfl_down(m[v], off);
            m[v] = merge(m[v], o);
        }
    if (lane == 0)
#pragma unroll
        for (int v = 0; v < V; ++v) sm[warp][v] = m[v];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            Moments acc = sm[0][v];
            for (int w = 1; w < kRedThreads / 32; ++w) acc = merge(acc, sm[w][v]);
            m[v] = acc;
        }
    }
}

// Per-thread running sums about a shift k (the thread's first value): n, sum (x - k) and
// sum (x - k)^2, turned into a (count, mean, M2) triple once at the end of the thread's range.
// No division per sample (an FP64 division is a dozen FP64 operations, on a part whose FP64 rate
// is a small fraction of its FP32 rate); the shift keeps the second sum free of the cancellation
// of raw moments.
struct ShiftSums { double n, k, s1, s2; };

__device__ __forceinline__ void add(ShiftSums& a, double x) {
    if (a.n == 0.0) a.k = x;
    const double d = x - a.k;
    a.n += 1.0;
    a.s1 += d;
    a.s2 = fma(d, d, a.s2);
}

__device__ __forceinline__ Moments moments_of(const ShiftSums& a) {
    if (a.n == 0.0) return Moments{0, 0, 0};
    const double md = a.s1 / a.n;
    return Moments{a.n, a.k + md, fmax(0.0, a.s2 - a.s1 * md)};
}

// the reference's per-sample terms (stats.py:42-48), one division per sample: h1 = 1 / (2 db),
// h2 = 1 / db^2
__device__ __forceinline__ void terms(const double* rho, const double* g, const double* gp,
                                      const double* gm, int64_t i, double h1, double h2, double& r,
                                      double& s1, double& s2) {
    const double rh = rho[i], gg = g[i];
    const double inv = 1.0 / rh;
    r = gg * inv;                                            // g / rho
    if (gp) {
        const double p = gp[i], m = gm[i];
        s1 = (p - m) * inv * h1;                             // (g+ - g-) / rho / (2 db)
        s2 = (p - 2.0 * gg + m) * inv * h2;                  // (g+ - 2g + g-) / rho / db^2
    } else {
        s1 = 0.0;
        s2 = 0.0;
    }
}

__global__ void terms_partial(const double* rho, const double* g, const double* gp, const double* gm,
                              int64_t X, double db, double* scratch) {
    const double h1 = 0.5 / db, h2 = 1.0 / (db * db);
    ShiftSums acc[3] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < X;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double r, s1, s2;
        terms(rho, g, gp, gm, i, h1, h2, r, s1, s2);
        add(acc[0], r);
        add(acc[1], s1);
        add(acc[2], s2);
    }
    Moments m[3] = {moments_of(acc[0]), moments_of(acc[1]), moments_of(acc[2])};
    block_merge<3>(m);
    if (threadIdx.x == 0)
        for (int v = 0; v < 3; ++v) {
            double* o = scratch + (static_cast<int64_t>(blockIdx.x) * 3 + v) * 3;
            o[0] = m[v].n; o[1] = m[v].mean; o[2] = m[v].m2;
        }
}

__global__ void jackknife_partial(const double* rho, const double* g, const double* gp,
                                  const double* gm, int64_t X, double db, double kT2,
                                  const double* totals, double* scratch) {
    const double Sr = totals[0], S1 = totals[1], S2 = totals[2];
    const double E0 = -S1 / Sr;
    const double h1 = 0.5 / db, h2 = 1.0 / (db * db), inv_kT2 = 1.0 / kT2;
    ShiftSums acc[2] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < X;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        double r, s1, s2;
        terms(rho, g, gp, gm, i, h1, h2, r, s1, s2);
        // f_E,i - E0 and f_C,i - C0 written without the cancellation of the direct differences:
        //   (S - x_i)/(S_r - r_i) - S/S_r = -(S_r x_i - S r_i) / (S_r (S_r - r_i))
        const double inv_den = 1.0 / (Sr * (Sr - r));
        const double dE = (Sr * s1 - S1 * r) * inv_den;
        const double dC = (-(Sr * s2 - S2 * r) * inv_den - dE * (2.0 * E0 + dE)) * inv_kT2;
        add(acc[0], dE);
        add(acc[1], dC);
    }
    Moments m[2] = {moments_of(acc[0]), moments_of(acc[1])};
    block_merge<2>(m);
    if (threadIdx.x == 0)
        for (int v = 0; v < 2; ++v) {
            double* o = scratch + (static_cast<int64_t>(blockIdx.x) * 2 + v) * 3;
            o[0] = m[v].n; o[1] = m[v].mean; o[2] = m[v].m2;
        }
}

template <int V>
__global__ void final_merge(const double* scratch, int nblocks, double* out) {
    Moments m[V];
#pragma unroll
    for (int v = 0; v < V; ++v) m[v] = Moments{0, 0, 0};
    // each thread merges a contiguous run of partials, then the block merges threads in order
    const int per = (nblocks + kRedThreads - 1) / kRedThreads;
    const int b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
    for (int b = b0; b < b1; ++b)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const double* s = scratch + (static_cast<int64_t>(b) * V + v) * 3;
            m[v] = merge(m[v], Moments{s[0], s[1], s[2]});
        }
    // ordered merge: lanes hold consecutive runs, shuffle-down merges keep the order
    block_merge<V>(m);
    if (threadIdx.x == 0) {
        out[0] = m[0].n;
#pragma unroll
        for (int v = 0; v < V; ++v) { out[1 + 2 * v] = m[v].mean; out[2 + 2 * v] = m[v].m2; }
    }
}

// ---- segmented variants: one independent reduction per model of a batched launch -----------
constexpr int kSegChunks = 32;

__global__ void terms_partial_seg(const double* rho, const double* g, const double* gp, const double* gm,
                                  const int64_t* seg, const double* dbeta, double* scratch) {
    const int m = blockIdx.y, c = blockIdx.x;
    const int64_t s0 = seg[m], s1 = seg[m + 1];
    const int64_t len = s1 - s0, chunk = (len + kSegChunks - 1) / kSegChunks;
    const int64_t c0 = s0 + c * chunk, c1 = min(s1, c0 + chunk);
    const double db = dbeta[m], h1 = 0.5 / db, h2 = 1.0 / (db * db);
    ShiftSums acc[3] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
        double r, a, b;
        terms(rho, g, gp, gm, i, h1, h2, r, a, b);
        add(acc[0], r);
        add(acc[1], a);
        add(acc[2], b);
    }
    Moments mo[3] = {moments_of(acc[0]), moments_of(acc[1]), moments_of(acc[2])};
    block_merge<3>(mo);
    if (threadIdx.x == 0)
        for (int v = 0; v < 3; ++v) {
            double* o = scratch + ((static_cast<int64_t>(m) * kSegChunks + c) * 3 + v) * 3;
            o[0] = mo[v].n; o[1] = mo[v].mean; o[2] = mo[v].m2;
        }
}

__global__ void jackknife_partial_seg(const double* rho, const double* g, const double* gp, const double* gm,
                                      const int64_t* seg, const double* dbeta, const double* kT2,
                                      const double* moments, double* scratch) {
    const int m = blockIdx.y, c = blockIdx.x;
    const int64_t s0 = seg[m], s1 = seg[m + 1];
    const int64_t len = s1 - s0, chunk = (len + kSegChunks - 1) / kSegChunks;
    const int64_t c0 = s0 + c * chunk, c1 = min(s1, c0 + chunk);
    const double* mm = moments + m * 7;
    const double Sr = mm[0] * mm[1], S1 = mm[0] * mm[3], S2 = mm[0] * mm[5];
    const double E0 = -S1 / Sr;
    const double db = dbeta[m], h1 = 0.5 / db, h2 = 1.0 / (db * db), inv_kT2 = 1.0 / kT2[m];
    ShiftSums acc[2] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int64_t i = c0 + threadIdx.x; i < c1; i += blockDim.x) {
        double r, a, b;
        terms(rho, g, gp, gm, i, h1, h2, r, a, b);
        const double inv_den = 1.0 / (Sr * (Sr - r));
        const double dE = (Sr * a - S1 * r) * inv_den;
        const double dC = (-(Sr * b - S2 * r) * inv_den - dE * (2.0 * E0 + dE)) * inv_kT2;
        add(acc[0], dE);
        add(acc[1], dC);
    }
    Moments mo[2] = {moments_of(acc[0]), moments_of(acc[1])};
    block_merge<2>(mo);
    if (threadIdx.x == 0)
        for (int v = 0; v < 2; ++v) {
            double* o = scratch + ((static_cast<int64_t>(m) * kSegChunks + c) * 2 + v) * 3;
            o[0] = mo[v].n; o[1] = mo[v].mean; o[2] = mo[v].m2;
        }
}

template <int V>
__global__ void final_merge_seg(const double* scratch, double* out) {
    const int m = blockIdx.x;
    if (threadIdx.x != 0) return;
    Moments acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = Moments{0, 0, 0};
    for (int c = 0; c < kSegChunks; ++c)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const double* s = scratch + ((static_cast<int64_t>(m) * kSegChunks + c) * V + v) * 3;
            acc[v] = merge(acc[v], Moments{s[0], s[1], s[2]});
        }
    double* o = out + m * (1 + 2 * V);
    o[0] = acc[0].n;
#pragma unroll
    for (int v = 0; v < V; ++v) { o[1 + 2 * v] = acc[v].mean; o[2 + 2 * v] = acc[v].m2; }
}

int nblocks_for(int64_t X) {
    int64_t nb = (X + kPerBlock - 1) / kPerBlock;
    if (nb < 1) nb = 1;
    if (nb > kMaxBlocks) nb = kMaxBlocks;
    return static_cast<int>(nb);
}

}  // namespace

extern "C" {

int64_t pbr_reduce_blocks(int64_t X) { return nblocks_for(X); }

int64_t pbr_reduce_segments_scratch(int32_t M) { return static_cast<int64_t>(M) * kSegChunks * 9; }

int pbr_reduce_terms_segments(const double* s_rho, const double* s_g, const double* s_gp, const double* s_gm,
                              const int64_t* seg, int32_t M, const double* delta_beta, double* scratch,
                              double* moments, void* stream) {
    if (!s_rho || !s_g || !seg || !delta_beta || !scratch || !moments || M < 1 || M > 65535) return PBR_ERR_ARG;
    if ((s_gp == nullptr) != (s_gm == nullptr)) return PBR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    terms_partial_seg<<<dim3(kSegChunks, M), kRedThreads, 0, st>>>(s_rho, s_g, s_gp, s_gm, seg, delta_beta, scratch);
    final_merge_seg<3><<<M, 32, 0, st>>>(scratch, moments);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int pbr_reduce_jackknife_segments(const double* s_rho, const double* s_g, const double* s_gp, const double* s_gm,
                                  const int64_t* seg, int32_t M, const double* delta_beta, const double* kB_T2,
                                  const double* moments, double* scratch, double* out, void* stream) {
    if (!s_rho || !s_g || !s_gp || !s_gm || !seg || !delta_beta || !kB_T2 || !moments || !scratch || !out ||
        M < 1 || M > 65535)
        return PBR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    jackknife_partial_seg<<<dim3(kSegChunks, M), kRedThreads, 0, st>>>(s_rho, s_g, s_gp, s_gm, seg, delta_beta,
                                                                       kB_T2, moments, scratch);
    final_merge_seg<2><<<M, 32, 0, st>>>(scratch, out);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int pbr_reduce_terms(const double* s_rho, const double* s_g, const double* s_gp,
                     const double* s_gm, int64_t X, double delta_beta, double* scratch,
                     double* moments, void* stream) {
    if (!s_rho || !s_g || !scratch || !moments || X < 1) return PBR_ERR_ARG;
    if ((s_gp == nullptr) != (s_gm == nullptr)) return PBR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = nblocks_for(X);
    terms_partial<<<nb, kRedThreads, 0, st>>>(s_rho, s_g, s_gp, s_gm, X, delta_beta, scratch);
    final_merge<3><<<1, kRedThreads, 0, st>>>(scratch, nb, moments);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int pbr_reduce_jackknife(const double* s_rho, const double* s_g, const double* s_gp,
                         const double* s_gm, int64_t X, double delta_beta, double kB_T2,
                         const double* totals, double* scratch, double* out, void* stream) {
    if (!s_rho || !s_g || !s_gp || !s_gm || !totals || !scratch || !out || X < 2) return PBR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = nblocks_for(X);
    jackknife_partial<<<nb, kRedThreads, 0, st>>>(s_rho, s_g, s_gp, s_gm, X, delta_beta, kB_T2,
                                                  totals, scratch);
    final_merge<2><<<1, kRedThreads, 0, st>>>(scratch, nb, out);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Allocation-free variant of pbr_reduce_terms.
//
// For callers that cannot allocate device memory: a plain FFI caller (ctypes from a job script,
// say) that has no GPU array library to allocate through, or a caller whose device memory is
// held by its own pool and that must not call cudaMalloc / cudaFree, which can synchronize the
// device.  The partial-sum scratch lives in this file-scope array instead of a caller buffer.
// Every device that loads the library keeps the array (kStaticScratchDoubles doubles, 72 KiB)
// until the process exits.
// ---------------------------------------------------------------------------------------------
#include <mutex>

namespace {

constexpr int kStaticBlocks = 1024;                                 // partial blocks held
constexpr int64_t kStaticMaxSamples = static_cast<int64_t>(kStaticBlocks) * kPerBlock;
constexpr int kStaticScratchDoubles = 9 * kStaticBlocks;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

std::mutex g_static_mutex;
double* g_static_addr[kMaxDevices] = {nullptr};

// Device address of g_static_scratch on the current device, looked up once per device and kept
// for the life of the process (a device reset that re-creates the context can move the array; the
// header tells callers not to use this entry point on a device after one).  In host code the
// symbol name is only a host-side stand-in for the array, so kernels must be given this address,
// never &g_static_scratch.
int static_scratch_address(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PBR_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (g_static_addr[dev] == nullptr) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || p == nullptr)
            return PBR_ERR_CUDA;
        g_static_addr[dev] = static_cast<double*>(p);
    }
    *out = g_static_addr[dev];
    return PBR_OK;
}

}  // namespace

extern "C" {

int64_t pbr_reduce_terms_static_max_samples(void) { return kStaticMaxSamples; }

int pbr_reduce_terms_static(const double* s_rho, const double* s_g, const double* s_gp,
                            const double* s_gm, int64_t X, double delta_beta, double* moments,
                            void* stream) {
    if (!s_rho || !s_g || !moments || X < 1) return PBR_ERR_ARG;
    if ((s_gp == nullptr) != (s_gm == nullptr)) return PBR_ERR_ARG;
    if (X > kStaticMaxSamples) return PBR_ERR_CAPACITY;
    double* scratch = nullptr;
    const int rc = static_scratch_address(&scratch);
    if (rc != PBR_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = nblocks_for(X);          // <= kStaticBlocks for X <= kStaticMaxSamples
    // every partial slot the merge reads is written by terms_partial first: nothing to clear
    terms_partial<<<nb, kRedThreads, 0, st>>>(s_rho, s_g, s_gp, s_gm, X, delta_beta, scratch);
    final_merge<3><<<1, kRedThreads, 0, st>>>(scratch, nb, moments);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

}  // extern "C"
