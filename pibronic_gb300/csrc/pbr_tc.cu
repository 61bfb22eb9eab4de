// pbr_tc.cu -- 5th-generation tensor-core (tcgen05) GEMM for sm_103a, written with inline PTX:
// operands staged in shared memory in the canonical no-swizzle K-major layout, one elected thread
// issues tcgen05.mma into a TMEM accumulator, completion is signalled through an mbarrier
// (tcgen05.commit), and the warps read the accumulator back with tcgen05.ld.
//
// pbr_tc_gemm: C[M][N] (FP32) = A[M][K] * B[N][K]^T for BF16 or TF32 operands, M % 128 == 0,
// N % 16 == 0 (16 <= N <= 256), K a multiple of the stage depth.  Every wait is bounded: on a
// timeout the CTA records PBR_ERR_CUDA in *status, skips the rest of its work, and still frees
// its TMEM.
#include <cstdint>

#include "pbr_common.cuh"

namespace {

constexpr int kTcThreads = 128;          // one warpgroup: warp w reads TMEM lanes 32w .. 32w+31
constexpr int kBM = 128;
constexpr int kStageBytesK = 128;        // bytes of K per stage (64 bf16 or 32 tf32)
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 64-bit shared-memory matrix descriptor: no swizzle, K-major, core matrices of 8 rows x 16 B;
// lbo = byte step between core matrices along K, sbo = byte step between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((addr & 0x3FFFF) >> 4);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;
    d |= static_cast<uint64_t>(1) << 46;            // descriptor version for sm_100 family
    return d;                                        // base offset 0, layout type 0 (no swizzle)
}

// 32-bit instruction descriptor: FP32 accumulator, both operands K-major, dense.
__host__ __device__ constexpr uint32_t instr_desc(int fmt, int M, int N) {
    return (1u << 4)                                 // accumulator format F32
         | (static_cast<uint32_t>(fmt) << 7)         // A format (1 = BF16, 2 = TF32)
         | (static_cast<uint32_t>(fmt) << 10)        // B format
         | (static_cast<uint32_t>(N >> 3) << 17)
         | (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

// bounded wait for the phase with the given parity; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

template <int FMT>
__device__ __forceinline__ void mma_issue(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    if constexpr (FMT == 1) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
            ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
            ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
    }
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(smem_u32(bar)) : "memory");
}

// 32 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Copy a rows x (kStageBytesK bytes) K-slice of a row-major matrix into the core-matrix layout:
// core (row group g, k group c) at ((g * KC) + c) * 128 bytes, 16 B per row inside the core.
__device__ __forceinline__ void stage_tile(const unsigned char* __restrict__ src, int64_t row_bytes, int rows,
                                           unsigned char* dst) {
    constexpr int KC = kStageBytesK / 16;            // core matrices along K per stage
    for (int i = threadIdx.x; i < rows * KC; i += blockDim.x) {
        const int row = i / KC, c = i - row * KC;
        const uint4 v = *reinterpret_cast<const uint4*>(src + row * row_bytes + c * 16);
        const int g = row >> 3, rr = row & 7;
        *reinterpret_cast<uint4*>(dst + ((g * KC + c) * 8 + rr) * 16) = v;
    }
}

template <int FMT>
__global__ void __launch_bounds__(kTcThreads) tc_gemm_kernel(const void* __restrict__ A, const void* __restrict__ B,
                                                             float* __restrict__ Cout, int M, int N, int K,
                                                             int ncols, int32_t* status) {
    constexpr int ESZ = (FMT == 1) ? 2 : 4;
    constexpr int KSTAGE = kStageBytesK / ESZ;          // elements of K per stage
    constexpr int KMMA = 32 / ESZ;                      // elements of K per tcgen05.mma
    extern __shared__ __align__(1024) unsigned char tsm[];
    unsigned char* sa = tsm;                            // 128 rows x 128 B
    unsigned char* sb = sa + kBM * kStageBytesK;        // N rows x 128 B
    uint64_t* bar = reinterpret_cast<uint64_t*>(sb + N * kStageBytesK);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = instr_desc(FMT, kBM, N);
    bool ok = true;
    uint32_t phase = 0;
    const unsigned char* Ab = static_cast<const unsigned char*>(A);
    const unsigned char* Bb = static_cast<const unsigned char*>(B);
    const int64_t a_row = static_cast<int64_t>(K) * ESZ, b_row = a_row;
    for (int k0 = 0; k0 < K && ok; k0 += KSTAGE) {
        stage_tile(Ab + static_cast<int64_t>(m0) * a_row + static_cast<int64_t>(k0) * ESZ, a_row, kBM, sa);
        stage_tile(Bb + static_cast<int64_t>(k0) * ESZ, b_row, N, sb);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            constexpr uint32_t LBO = 128, SBO = (kStageBytesK / 16) * 128;
#pragma unroll
            for (int kk = 0; kk < KSTAGE; kk += KMMA) {
                const uint32_t off = static_cast<uint32_t>(kk * ESZ / 16) * 128;   // cores along K
                mma_issue<FMT>(tmem, smem_desc(smem_u32(sa) + off, LBO, SBO), smem_desc(smem_u32(sb) + off, LBO, SBO),
                               idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(bar);
        }
        __syncwarp();
        const bool done = mbar_wait(bar, phase);
        asm volatile("tcgen05.fence::after_thread_sync;");
        // block-uniform outcome; the operands of the next stage overwrite the shared tiles
        ok = __syncthreads_and(done) != 0;
        if (ok) phase ^= 1u;
    }
    if (!ok) {
        mbar_wait(bar, phase);    // drain the MMAs still in flight (bounded) before freeing TMEM
        if (status && threadIdx.x == 0) atomicMax(status, PBR_ERR_CUDA);
    } else {
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < N; c0 += 32) {
            float v[32];
            tmem_ld32(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0), v);
            if (row < M)
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (c0 + i < N) Cout[static_cast<int64_t>(row) * N + c0 + i] = v[i];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace

extern "C" int pbr_tc_gemm(int32_t fmt, const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K,
                           int32_t* status, void* stream) {
    if (!A || !B || !C || (fmt != 1 && fmt != 2)) return PBR_ERR_ARG;
    const int esz = fmt == 1 ? 2 : 4;
    const int kstage = kStageBytesK / esz;
    if (M < kBM || M % kBM != 0 || N < 16 || N > 256 || N % 16 != 0 || K < kstage || K % kstage != 0)
        return PBR_ERR_ARG;
    // global row starts must be 16-byte aligned for the staging loads
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return PBR_ERR_ARG;
    int ncols = 32;
    while (ncols < N) ncols <<= 1;
    const int bytes = (kBM + N) * kStageBytesK + 16;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // at least 80 KB of shared memory per CTA caps residency at two CTAs (<= 512 TMEM columns)
    const int smem = bytes < 80 * 1024 ? 80 * 1024 : bytes;
    if (fmt == 1) {
        if (cudaFuncSetAttribute(tc_gemm_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        tc_gemm_kernel<1><<<M / kBM, kTcThreads, smem, st>>>(A, B, C, M, N, K, ncols, status);
    } else {
        if (cudaFuncSetAttribute(tc_gemm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        tc_gemm_kernel<2><<<M / kBM, kTcThreads, smem, st>>>(A, B, C, M, N, K, ncols, status);
    }
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}
// ---------------------------------------------------------------------------------------------
// The quadratic coupling contraction on tensor cores (pimc.py:1147, the 'acef,debc,abdf->afbc'
// einsum):  Vq[row][pr] = sum_{k=(d>=e)} (q_d q_e)[row] * Qp[pr][k]   for row = sample * P + bead,
// pr = pair_index(b, c), k = pair_index(d, e) and Qp[pr][k] the symmetrised 1/2 Q couplings.
//
// TF32 with a hi/lo split of both operands: three MMAs per K step (hi*hi + hi*lo + lo*hi) with
// FP32 accumulation in TMEM keep about 21 bits of every product, the accuracy of the FP32 FMA
// form.  The A operand (pair products of the row's bead coordinates) is generated into shared
// memory stage by stage; the B operand (Qp hi and lo, [A2P][N2P] K-major, packed on the device by
// pbr_tc_pack_quadratic) is copied per stage from L2.  Two stage buffers: the threads generate
// stage s+1 while the tensor core multiplies stage s.  A CTA is 256 threads on 128 rows (two
// threads per row, one per half of the stage's K slice); TMEM lane r holds row r.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int kQThreads = 256;
constexpr int kQStageK = 32;                          // TF32 elements of K per stage (128 B)
constexpr int kQStageBytesA = kBM * kStageBytesK;     // one 128-row operand part of one stage

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

struct QuadSmem {
    int a, b, q, pairs, bar, total;
    __host__ __device__ QuadSmem(int N, int N2P, int A2P) {
        int o = 0;
        a = o;     o += 2 * 2 * kQStageBytesA;                // [buffer][hi, lo] A stages
        b = o;     o += 2 * 2 * A2P * kStageBytesK;           // [buffer][hi, lo] B stages
        q = o;     o += kBM * (N | 1) * 4;                    // bead coordinates, odd row stride
        pairs = o; o += ((N2P * 4 + 15) / 16) * 16;           // (d, e) of every K index
        bar = o;   o += 32;                                   // two mbarriers + the TMEM slot
        total = o;
    }
};

__global__ void __launch_bounds__(kQThreads) tc_quadratic_kernel(
        const float* __restrict__ q, int64_t X, int N, int P, int N2, int N2P, int A2P,
        const float* __restrict__ b_hi, const float* __restrict__ b_lo, float* __restrict__ vq, int ncols,
        int32_t* status) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    const QuadSmem L(N, N2P, A2P);
    unsigned char* sa = tsm + L.a;
    unsigned char* sb = tsm + L.b;
    float* sq = reinterpret_cast<float*>(tsm + L.q);
    int16_t* spair = reinterpret_cast<int16_t*>(tsm + L.pairs);
    uint64_t* bar = reinterpret_cast<uint64_t*>(tsm + L.bar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
    const int NS = N | 1;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int BSTAGE = A2P * kStageBytesK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) { mbar_init(bar, 1); mbar_init(bar + 1, 1); }
    for (int d = tid; d < N; d += kQThreads)
        for (int e = 0; e <= d; ++e) {
            const int k = d * (d + 1) / 2 + e;
            spair[2 * k] = static_cast<int16_t>(d);
            spair[2 * k + 1] = static_cast<int16_t>(e);
        }
    for (int k = N2 + tid; k < N2P; k += kQThreads) { spair[2 * k] = 0; spair[2 * k + 1] = 0; }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = instr_desc(2, kBM, A2P);
    constexpr uint32_t LBO = 128, SBO = (kStageBytesK / 16) * 128;
    uint32_t phase = 0u;                              // bit b: parity of buffer b's next commit
    uint32_t pend = 0u;                               // bit b: a commit of buffer b not yet waited for
    bool ok = true;
    const int row_l = tid & (kBM - 1), half = tid >> 7;   // this thread's row and K half
    const int64_t rows = X * P;
    const int64_t tiles = (rows + kBM - 1) / kBM;
    const int nst = N2P / kQStageK;

    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t r0 = tile * kBM;
        for (int i = tid; i < kBM * N; i += kQThreads) {
            const int rr = i % kBM, j = i / kBM;
            const int64_t row = r0 + rr;
            float v = 0.f;
            if (row < rows) {
                const int64_t x = row / P;
                const int p = static_cast<int>(row - x * P);
                v = q[(x * N + j) * P + p];
            }
            sq[rr * NS + j] = v;
        }
        __syncthreads();
        const float* myq = sq + row_l * NS;
        for (int st = 0; st < nst; ++st) {
            const int bf = st & 1;
            if (pend & (1u << bf)) {               // the MMAs of stage st-2 read this buffer
                if (ok) ok = mbar_wait(bar + bf, (phase >> bf) & 1u);
                phase ^= 1u << bf;
                pend &= ~(1u << bf);
            }
            unsigned char* ahi = sa + bf * 2 * kQStageBytesA;
            unsigned char* alo = ahi + kQStageBytesA;
            unsigned char* bhi = sb + bf * 2 * BSTAGE;
            unsigned char* blo = bhi + BSTAGE;
            const int k0 = st * kQStageK;
            {
                const int g = row_l >> 3, rr = row_l & 7;
#pragma unroll
                for (int cc = 0; cc < kQStageK / 8; ++cc) {
                    const int c = half * (kQStageK / 8) + cc;       // 16-byte core column 0..7
                    float hi[4], lo[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int k = k0 + 4 * c + u;
                        const uint32_t de = *reinterpret_cast<const uint32_t*>(spair + 2 * k);
                        const float pr = myq[de & 0xFFFF] * myq[de >> 16];
                        hi[u] = tf32_rna(pr);
                        lo[u] = tf32_rna(pr - hi[u]);
                    }
                    const int off = ((g * (kStageBytesK / 16) + c) * 8 + rr) * 16;
                    *reinterpret_cast<float4*>(ahi + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                    *reinterpret_cast<float4*>(alo + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
                }
            }
            for (int i = tid; i < A2P * (kStageBytesK / 16); i += kQThreads) {
                const int pr = i / (kStageBytesK / 16), c = i - pr * (kStageBytesK / 16);
                const int off = (((pr >> 3) * (kStageBytesK / 16) + c) * 8 + (pr & 7)) * 16;
                const int64_t src = static_cast<int64_t>(pr) * N2P + k0 + 4 * c;
                *reinterpret_cast<float4*>(bhi + off) = __ldg(reinterpret_cast<const float4*>(b_hi + src));
                *reinterpret_cast<float4*>(blo + off) = __ldg(reinterpret_cast<const float4*>(b_lo + src));
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0 && ok) {
                asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
                for (int kk = 0; kk < kQStageK; kk += 8) {
                    const uint32_t off = static_cast<uint32_t>(kk * 4 / 16) * 128;
                    const uint64_t dah = smem_desc(smem_u32(ahi) + off, LBO, SBO);
                    const uint64_t dal = smem_desc(smem_u32(alo) + off, LBO, SBO);
                    const uint64_t dbh = smem_desc(smem_u32(bhi) + off, LBO, SBO);
                    const uint64_t dbl = smem_desc(smem_u32(blo) + off, LBO, SBO);
                    mma_issue<2>(tmem, dah, dbh, idesc, (st > 0 || kk > 0) ? 1u : 0u);
                    mma_issue<2>(tmem, dah, dbl, idesc, 1u);
                    mma_issue<2>(tmem, dal, dbh, idesc, 1u);
                }
            }
            if (tid == 0) mma_commit(bar + bf);   // arrives once the MMAs issued so far complete
            pend |= 1u << bf;
        }
        // drain both buffers: the accumulator is final once the last commit has arrived
#pragma unroll
        for (int bf = 0; bf < 2; ++bf)
            if (pend & (1u << bf)) {
                if (ok) ok = mbar_wait(bar + bf, (phase >> bf) & 1u);
                phase ^= 1u << bf;
                pend &= ~(1u << bf);
            }
        asm volatile("tcgen05.fence::after_thread_sync;");
        ok = __syncthreads_and(ok) != 0;
        if (!ok) break;
        {
            const int lg = warp & 3, ch = warp >> 2;
            const int64_t row = r0 + lg * 32 + lane;
            for (int c0 = ch * 32; c0 < A2P; c0 += 64) {
                float v[32];
                tmem_ld32(tmem + (static_cast<uint32_t>(lg * 32) << 16) + static_cast<uint32_t>(c0), v);
                if (row < rows) {
                    float* dst = vq + row * A2P + c0;
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        if (c0 + i < A2P) *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncthreads();
    }
    if (!ok) {
        // bounded drain of MMAs still in flight before the TMEM is freed
        for (int bf = 0; bf < 2; ++bf)
            if (pend & (1u << bf)) mbar_wait(bar + bf, (phase >> bf) & 1u);
        if (status && tid == 0) atomicMax(status, PBR_ERR_CUDA);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Qp (FP32 or FP64 [N2][A2], row k = pair_index(d, e)) -> TF32 hi / lo, [A2P][N2P] K-major, zero padded
template <typename T>
__global__ void tc_pack_kernel(const T* __restrict__ qq, int N2, int A2, int N2P, int A2P, float* __restrict__ bh,
                               float* __restrict__ bl) {
    const int64_t n = static_cast<int64_t>(A2P) * N2P;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int pr = static_cast<int>(i / N2P), k = static_cast<int>(i - static_cast<int64_t>(pr) * N2P);
        const float x = (pr < A2 && k < N2) ? static_cast<float>(qq[static_cast<int64_t>(k) * A2 + pr]) : 0.f;
        const float h = tf32_rna(x);
        bh[i] = h;
        bl[i] = tf32_rna(x - h);
    }
}

}  // namespace

namespace pbr {

int tc_quadratic_cols(int A) { return (A * (A + 1) / 2 + 15) / 16 * 16; }
int tc_quadratic_kdim(int N) { return (N * (N + 1) / 2 + kQStageK - 1) / kQStageK * kQStageK; }

int tc_quadratic_launch(const float* q, int64_t X, int N, int P, int A2P, const float* b_hi, const float* b_lo,
                        int N2P, float* vq, int32_t* status, cudaStream_t stream) {
    if (!q || !b_hi || !b_lo || !vq || X < 0 || N < 1 || N > 64 || P < 1) return PBR_ERR_ARG;
    const int N2 = N * (N + 1) / 2;
    if (N2P < N2 || N2P % kQStageK != 0 || A2P < 16 || A2P > 256 || A2P % 16 != 0) return PBR_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(b_hi) | reinterpret_cast<uintptr_t>(b_lo) | reinterpret_cast<uintptr_t>(vq)) & 15)
        return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    int ncols = 32;
    while (ncols < A2P) ncols <<= 1;
    const QuadSmem L(N, N2P, A2P);
    if (L.total > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    static int configured = 0;
    if (L.total > configured) {
        if (cudaFuncSetAttribute(tc_quadratic_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = 227 * 1024;
    }
    int dev = 0, sms = 0, occ = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tc_quadratic_kernel, kQThreads, L.total));
    if (occ < 1) return PBR_ERR_UNSUPPORTED;
    if (occ * ncols > 512) occ = 512 / ncols;          // TMEM columns of the resident CTAs
    const int64_t tiles = (X * P + kBM - 1) / kBM;
    const int grid = static_cast<int>(tiles < static_cast<int64_t>(occ) * sms ? tiles : static_cast<int64_t>(occ) * sms);
    tc_quadratic_kernel<<<grid, kQThreads, L.total, stream>>>(q, X, N, P, N2, N2P, A2P, b_hi, b_lo, vq, ncols,
                                                              status);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int tc_pack_launch(const void* qq, int precision, int N, int A, float* b_hi, float* b_lo, cudaStream_t stream) {
    if (!qq || !b_hi || !b_lo || N < 1 || N > 64 || A < 1 || A > 22) return PBR_ERR_ARG;
    const int N2 = N * (N + 1) / 2, A2 = A * (A + 1) / 2;
    const int N2P = tc_quadratic_kdim(N), A2P = tc_quadratic_cols(A);
    const int64_t n = static_cast<int64_t>(A2P) * N2P;
    const int grid = static_cast<int>((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    if (precision == 32)
        tc_pack_kernel<float><<<grid, 256, 0, stream>>>(static_cast<const float*>(qq), N2, A2, N2P, A2P, b_hi, b_lo);
    else if (precision == 64)
        tc_pack_kernel<double><<<grid, 256, 0, stream>>>(static_cast<const double*>(qq), N2, A2, N2P, A2P, b_hi, b_lo);
    else
        return PBR_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

}  // namespace pbr

extern "C" {

int pbr_tc_quadratic_dims(int32_t N, int32_t A, int32_t* n2p, int32_t* a2p) {
    if (N < 1 || N > 64 || A < 1 || A > 22 || !n2p || !a2p) return PBR_ERR_ARG;
    *n2p = pbr::tc_quadratic_kdim(N);
    *a2p = pbr::tc_quadratic_cols(A);
    return PBR_OK;
}

int pbr_tc_pack_quadratic(const void* vib_qq, int32_t precision, int32_t N, int32_t A, float* b_hi, float* b_lo,
                          void* stream) {
    return pbr::tc_pack_launch(vib_qq, precision, N, A, b_hi, b_lo, static_cast<cudaStream_t>(stream));
}

int pbr_tc_quadratic(const float* q, int64_t X, int32_t N, int32_t P, int32_t A, const float* b_hi,
                     const float* b_lo, float* vq, int32_t* status, void* stream) {
    if (A < 1 || A > 22) return PBR_ERR_ARG;
    return pbr::tc_quadratic_launch(q, X, N, P, pbr::tc_quadratic_cols(A), b_hi, b_lo, pbr::tc_quadratic_kdim(N),
                                    vq, status, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
