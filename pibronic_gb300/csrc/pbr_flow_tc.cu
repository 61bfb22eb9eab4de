// pbr_flow_tc.cu -- the learned proposal's coupling layers on the 5th-generation tensor cores, for
// the sampling direction.  No counterpart in the reference (see pbr_flow.cu).
//
// One layer maps y -> y' with y'_b = y_b exp(s(y_a)) + t(y_a) on the layer's index sets a, b;
// (s, t) = head(tanh(W2^T tanh(W1^T y_a + b1) + b2)), s = 2 tanh(raw / 2).  Per tile of 128 samples
// the three products are tcgen05.mma kind::f16 GEMMs with BF16 operands (M = 128 samples, the
// weights as the N side) and FP32 accumulators in TMEM; the activations go back through shared
// memory as BF16 A operands.  The coupling update, exp(s) and the log-determinant (the sum of s)
// stay in FP32, accumulated into FP64 per sample.
//
// Exactness: whatever rounding the BF16 network applies, y_b' depends on y_a only through the s
// and t it computed, and y_a passes unchanged, so log |det dy'/dy| is exactly the sum of those s.
// The proposal density computed alongside the samples is therefore the density of the map that
// produced them, and g / q stays unbiased; the BF16 network only moves the map a little away from
// the FP32 one that training optimised.
//
// Layout: the CTA holds the layer's packed weights (pbr_flow_tc_pack) and runs one or two
// warpgroups, each an independent pipeline over its own tiles: thread r of a warpgroup owns sample
// row r (its TMEM lane), thread 0 issues the MMAs and commits them to the warpgroup's mbarrier.
// Every wait is bounded; a timeout records PBR_ERR_CUDA and the warpgroup leaves its tile loop.
#include <cuda_bf16.h>

#include "pbr_common.cuh"
#include "pbr_tcgen05.cuh"

namespace {

constexpr int kRows = 128;                  // samples per tile (the MMA's M)
constexpr float kKappaTc = 2.0f;            // s = kKappa tanh(raw / kKappa), as in pbr_flow.cu

__host__ __device__ inline int up(int x, int a) { return (x + a - 1) / a * a; }

// Packed layer (pbr_flow_tc_pack), in bytes from the start:
//   W1t [H][K1], W2t [H][H], W3t [N3][H] BF16 B operands (K-major core layout: core (n, k) at
//   ((n / 8) * (K / 8) + k / 8) * 8 + n % 8 in 16-byte units, element k % 8 within), with
//   K1 = I rounded up to 16 and N3 = 2J rounded up to 32; the head's rows interleave s and t
//   (row 2j = s_j, row 2j + 1 = t_j);
//   then b1 [H], b2 [H], b3 [N3] (interleaved like the rows) as FP32.
struct TcLayerDims {
    int D, I, J, H, K1, N3;
    int w1, w2, w3, b1, b2, b3, bytes;
    __host__ __device__ TcLayerDims(int D_, int I_, int J_, int H_) : D(D_), I(I_), J(J_), H(H_) {
        K1 = up(I, 16);
        N3 = up(2 * J, 32);
        int o = 0;
        w1 = o; o += H * K1 * 2;
        w2 = o; o += H * H * 2;
        w3 = o; o += N3 * H * 2;
        b1 = o; o += H * 4;
        b2 = o; o += H * 4;
        b3 = o; o += N3 * 4;
        bytes = up(o, 16);
    }
};

__host__ __device__ inline bool tc_supported(int D, int I, int J, int H) {
    return D >= 2 && I >= 1 && J >= 1 && I + J == D && H >= 32 && H <= 128 && H % 32 == 0 && I <= 128 &&
           2 * J <= 256;
}

// 16-byte unit of core-layout element (n, k) in a K-major operand of K columns
__host__ __device__ inline int core_unit(int n, int k, int K) { return ((n >> 3) * (K >> 3) + (k >> 3)) * 8 + (n & 7); }

// shared-memory plan of the forward kernel, in bytes
struct TcFwdSmem {
    int wg, Dp, wts, idx, abuf, ys, bars, total;
    __host__ __device__ TcFwdSmem(const TcLayerDims& L, int nwg) {
        wg = nwg;
        Dp = L.D | 1;                       // odd row stride of the y tile: conflict-free row reads
        int o = 0;
        wts = o;  o += L.bytes;
        idx = o;  o += up((L.K1 + L.J) * 4, 16);
        abuf = o; o += nwg * kRows * (L.K1 > L.H ? L.K1 : L.H) * 2;
        ys = o;   o += up(nwg * kRows * Dp * 4, 16);
        bars = o; o += 16 * nwg + 16;       // one mbarrier and an error flag per warpgroup, TMEM slot
        total = o;
    }
};

template <typename T>
__global__ void flow_tc_pack_kernel(int D, int I, int J, int H, const T* __restrict__ W1, const T* __restrict__ b1,
                                    const T* __restrict__ W2, const T* __restrict__ b2, const T* __restrict__ W3,
                                    const T* __restrict__ b3, unsigned char* __restrict__ out) {
    const TcLayerDims L(D, I, J, H);
    __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(out + L.w1);
    __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(out + L.w2);
    __nv_bfloat16* w3 = reinterpret_cast<__nv_bfloat16*>(out + L.w3);
    float* fb1 = reinterpret_cast<float*>(out + L.b1);
    float* fb2 = reinterpret_cast<float*>(out + L.b2);
    float* fb3 = reinterpret_cast<float*>(out + L.b3);
    const int n1 = H * L.K1, n2 = H * H, n3 = L.N3 * H;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n1 + n2 + n3 + 2 * H + L.N3; i += gridDim.x * blockDim.x) {
        if (i < n1) {                                   // W1t (n = h, k = input i)
            const int n = i / L.K1, k = i - n * L.K1;
            const float v = k < I ? static_cast<float>(W1[k * H + n]) : 0.f;
            w1[core_unit(n, k, L.K1) * 8 + (k & 7)] = __float2bfloat16_rn(v);
        } else if (i < n1 + n2) {                       // W2t (n = h_out, k = h_in)
            const int e = i - n1, n = e / H, k = e - n * H;
            w2[core_unit(n, k, H) * 8 + (k & 7)] = __float2bfloat16_rn(static_cast<float>(W2[k * H + n]));
        } else if (i < n1 + n2 + n3) {                  // W3t (n = 2j: s_j, 2j + 1: t_j; k = h)
            const int e = i - n1 - n2, n = e / H, k = e - n * H;
            const int j = n >> 1, col = (n & 1) ? J + j : j;
            const float v = j < J ? static_cast<float>(W3[k * (2 * J) + col]) : 0.f;
            w3[core_unit(n, k, H) * 8 + (k & 7)] = __float2bfloat16_rn(v);
        } else {
            const int e = i - n1 - n2 - n3;
            if (e < H) fb1[e] = static_cast<float>(b1[e]);
            else if (e < 2 * H) fb2[e - H] = static_cast<float>(b2[e - H]);
            else {
                const int n = e - 2 * H, j = n >> 1;
                fb3[n] = j < J ? static_cast<float>(b3[(n & 1) ? J + j : j]) : 0.f;
            }
        }
    }
}

// named barrier of one warpgroup (ids 1, 2; id 0 is __syncthreads)
__device__ __forceinline__ void wg_sync(int wg) {
    asm volatile("bar.sync %0, 128;" ::"r"(1 + wg) : "memory");
}

// this thread's row of an activation tile in the A-operand core layout, from 32 FP32 values at
// columns c0 .. c0 + 31 (four 16-byte stores)
__device__ __forceinline__ void store_bf16_row32(unsigned char* a, int row, int c0, int K, const float (&v)[32]) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        uint4 w;
        uint32_t* u = reinterpret_cast<uint32_t*>(&w);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[8 * c + 2 * p], v[8 * c + 2 * p + 1]);
            u[p] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(a + core_unit(row, c0 + 8 * c, K) * 16) = w;
    }
}

// issue one GEMM: D (TMEM) = A [128][K] x B [N][K]^T, both BF16 in the core layout, K / 16 MMAs
__device__ __forceinline__ void issue_gemm(uint32_t d, const unsigned char* a, const unsigned char* b, int K, int N) {
    const uint32_t idesc = instr_desc(1, kRows, N);
    const uint32_t sbo = static_cast<uint32_t>(K / 8) * 128;
    for (int k = 0; k < K; k += 16) {
        const uint32_t off = static_cast<uint32_t>(k / 8) * 128;
        mma_issue<1>(d, smem_desc(smem_u32(a) + off, 128, sbo), smem_desc(smem_u32(b) + off, 128, sbo), idesc,
                     k > 0 ? 1u : 0u);
    }
}

__global__ void __launch_bounds__(256, 1) flow_tc_forward_kernel(int D, int I, int J, int H, int nwg,
                                                                    const unsigned char* __restrict__ packed,
                                                                    const int32_t* __restrict__ idx_a,
                                                                    const int32_t* __restrict__ idx_b, int64_t X,
                                                                    float* __restrict__ y, double* __restrict__ logdet,
                                                                    int32_t* status) {
    extern __shared__ __align__(1024) unsigned char fsm[];
    const TcLayerDims L(D, I, J, H);
    const TcFwdSmem S(L, nwg);
    const int tid = threadIdx.x, wg = tid >> 7, r = tid & (kRows - 1);
    const int K1 = L.K1, N3 = L.N3, Dp = S.Dp;
    unsigned char* w = fsm + S.wts;
    int32_t* sidx = reinterpret_cast<int32_t*>(fsm + S.idx);           // [K1] idx_a (-1 pad), [J] idx_b
    unsigned char* abuf = fsm + S.abuf + wg * kRows * (K1 > H ? K1 : H) * 2;
    float* ys = reinterpret_cast<float*>(fsm + S.ys) + wg * kRows * Dp;
    uint64_t* bar = reinterpret_cast<uint64_t*>(fsm + S.bars) + 2 * wg;
    volatile int* err = reinterpret_cast<volatile int*>(bar + 1);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(fsm + S.bars + 16 * nwg);
    const int ncols = 256 * nwg;

    // the layer's weights and index sets -> shared memory (16-byte copies), TMEM, barriers
    for (int i = tid; i < L.bytes / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(w)[i] = reinterpret_cast<const uint4*>(packed)[i];
    for (int i = tid; i < K1 + J; i += blockDim.x) sidx[i] = i < K1 ? (i < I ? idx_a[i] : -1) : idx_b[i - K1];
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (r == 0) {
        mbar_init(bar, 1);
        *err = 0;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");       // weights: generic -> async proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tbase = *tslot + static_cast<uint32_t>(256 * wg);
    const uint32_t lanes = static_cast<uint32_t>(((tid >> 5) & 3) * 32) << 16;  // this warp's TMEM lanes
    const float* fb1 = reinterpret_cast<const float*>(w + L.b1);
    const float* fb2 = reinterpret_cast<const float*>(w + L.b2);
    const float* fb3 = reinterpret_cast<const float*>(w + L.b3);
    uint32_t phase = 0;
    bool pending = false;                  // a commit not yet waited for (drained on an error)

    auto gemm_and_wait = [&](uint32_t d, const unsigned char* a, const unsigned char* b, int K, int N) -> bool {
        if (r == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            issue_gemm(d, a, b, K, N);
            mma_commit(bar);
        }
        pending = true;
        const bool ok = mbar_wait(bar, phase);
        if (!ok) *err = 1;
        else pending = false;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        wg_sync(wg);
        return *err == 0;
    };

    const int64_t ntiles = (X + kRows - 1) / kRows;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * nwg + wg; t < ntiles;
         t += static_cast<int64_t>(gridDim.x) * nwg) {
        const int64_t x0 = t * kRows;
        const int rows = static_cast<int>(X - x0 < kRows ? X - x0 : kRows);
        // ---- the tile's y rows -> shared memory (coalesced), rows past X zero ----
        const float* yg = y + x0 * D;
        for (int i = r; i < kRows * D; i += kRows) {
            const int rr = i / D, c = i - rr * D;
            ys[rr * Dp + c] = rr < rows ? yg[i] : 0.f;
        }
        wg_sync(wg);
        // ---- A1 = y_a (BF16, K1 columns, zero past I) ----
        for (int c0 = 0; c0 < K1; c0 += 32) {
            float v[32];
#pragma unroll
            for (int u = 0; u < 32; ++u) {
                const int k = c0 + u;
                v[u] = (k < K1 && sidx[k] >= 0) ? ys[r * Dp + sidx[k]] : 0.f;
            }
            if (c0 + 32 <= K1) {
                store_bf16_row32(abuf, r, c0, K1, v);
            } else {                                   // K1 = 16 mod 32: two of the four cores
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    uint4 q4;
                    uint32_t* u4 = reinterpret_cast<uint32_t*>(&q4);
#pragma unroll
                    for (int p = 0; p < 4; ++p) {
                        const __nv_bfloat162 h = __floats2bfloat162_rn(v[8 * c + 2 * p], v[8 * c + 2 * p + 1]);
                        u4[p] = *reinterpret_cast<const uint32_t*>(&h);
                    }
                    *reinterpret_cast<uint4*>(abuf + core_unit(r, c0 + 8 * c, K1) * 16) = q4;
                }
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        wg_sync(wg);
        // ---- h1 = tanh(y_a W1 + b1) ----
        if (!gemm_and_wait(tbase, abuf, w + L.w1, K1, H)) break;
        for (int c0 = 0; c0 < H; c0 += 32) {
            float v[32];
            tmem_ld32(tbase + lanes + static_cast<uint32_t>(c0), v);
#pragma unroll
            for (int u = 0; u < 32; ++u) v[u] = tanhf(v[u] + fb1[c0 + u]);
            store_bf16_row32(abuf, r, c0, H, v);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        wg_sync(wg);
        // ---- h2 = tanh(h1 W2 + b2) ----
        if (!gemm_and_wait(tbase + static_cast<uint32_t>(H), abuf, w + L.w2, H, H)) break;
        for (int c0 = 0; c0 < H; c0 += 32) {
            float v[32];
            tmem_ld32(tbase + lanes + static_cast<uint32_t>(H + c0), v);
#pragma unroll
            for (int u = 0; u < 32; ++u) v[u] = tanhf(v[u] + fb2[c0 + u]);
            store_bf16_row32(abuf, r, c0, H, v);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
        wg_sync(wg);
        // ---- (s, t) = head(h2 W3 + b3); y_b' = y_b exp(s) + t; log-det += sum s ----
        if (!gemm_and_wait(tbase, abuf, w + L.w3, H, N3)) break;
        float ssum = 0.f;
        for (int c0 = 0; c0 < N3; c0 += 32) {
            float v[32];
            tmem_ld32(tbase + lanes + static_cast<uint32_t>(c0), v);
#pragma unroll
            for (int p = 0; p < 16; ++p) {
                const int j = c0 / 2 + p;
                if (j < J) {
                    const float s = kKappaTc * tanhf((v[2 * p] + fb3[2 * j]) / kKappaTc);
                    const float tt = v[2 * p + 1] + fb3[2 * j + 1];
                    float* yb = ys + r * Dp + sidx[K1 + j];
                    *yb = fmaf(*yb, __expf(s), tt);
                    ssum += s;
                }
            }
        }
        if (r < rows) logdet[x0 + r] += static_cast<double>(ssum);
        asm volatile("tcgen05.fence::before_thread_sync;");
        wg_sync(wg);
        // ---- the tile's y rows back (coalesced) ----
        float* yo = y + x0 * D;
        for (int i = r; i < rows * D; i += kRows) {
            const int rr = i / D, c = i - rr * D;
            yo[i] = ys[rr * Dp + c];
        }
        wg_sync(wg);
    }
    if (pending && r == 0) mbar_wait(bar, phase ^ 1u);      // bounded drain after an error
    if (*err && r == 0 && status) atomicMax(status, PBR_ERR_CUDA);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (tid < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tslot), "r"(ncols));
}

}  // namespace

extern "C" {

int64_t pbr_flow_tc_packed_bytes(int32_t D, int32_t I, int32_t J, int32_t H) {
    if (!tc_supported(D, I, J, H)) return -1;
    const TcLayerDims L(D, I, J, H);
    if (TcFwdSmem(L, 1).total > 227 * 1024) return -1;      // weights + one tile do not fit
    return L.bytes;
}

int pbr_flow_tc_pack(const pbr_flow_layer* layer, void* packed, void* stream) {
    if (!layer || !packed) return PBR_ERR_ARG;
    const pbr_flow_layer& l = *layer;
    if (!tc_supported(l.D, l.I, l.J, l.H)) return PBR_ERR_UNSUPPORTED;
    if (!l.W1 || !l.b1 || !l.W2 || !l.b2 || !l.W3 || !l.b3 || (reinterpret_cast<uintptr_t>(packed) & 15))
        return PBR_ERR_ARG;
    const TcLayerDims L(l.D, l.I, l.J, l.H);
    const int n = l.H * L.K1 + l.H * l.H + L.N3 * l.H + 2 * l.H + L.N3;
    flow_tc_pack_kernel<float><<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        l.D, l.I, l.J, l.H, l.W1, l.b1, l.W2, l.b2, l.W3, l.b3, static_cast<unsigned char*>(packed));
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int pbr_flow_tc_forward(const pbr_flow_layer* layer, const void* packed, int64_t X, float* y, double* logdet,
                        int32_t* status, void* stream) {
    if (!layer || !packed || !y || !logdet || X < 0) return PBR_ERR_ARG;
    const pbr_flow_layer& l = *layer;
    if (!tc_supported(l.D, l.I, l.J, l.H)) return PBR_ERR_UNSUPPORTED;
    if (!l.idx_a || !l.idx_b || (reinterpret_cast<uintptr_t>(packed) & 15)) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const TcLayerDims L(l.D, l.I, l.J, l.H);
    int nwg = 2;
    if (TcFwdSmem(L, 2).total > 227 * 1024) nwg = 1;
    const TcFwdSmem S(L, nwg);
    if (S.total > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    static int configured = 0;
    if (S.total > configured) {
        if (cudaFuncSetAttribute(flow_tc_forward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = 227 * 1024;
    }
    int dev = 0, sms = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // one CTA per SM (its TMEM columns are 256 per warpgroup): at least half the shared memory
    const int smem = S.total > 116 * 1024 ? S.total : 116 * 1024;
    const int64_t tiles = (X + kRows - 1) / kRows;
    const int64_t need = (tiles + nwg - 1) / nwg;
    const int grid = static_cast<int>(need < sms ? need : sms);
    flow_tc_forward_kernel<<<grid, 128 * nwg, smem, static_cast<cudaStream_t>(stream)>>>(
        l.D, l.I, l.J, l.H, nwg, static_cast<const unsigned char*>(packed), l.idx_a, l.idx_b, X, y, logdet,
        status);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

}  // extern "C"
