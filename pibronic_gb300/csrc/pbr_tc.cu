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
        ok = mbar_wait(bar, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;");
        __syncthreads();          // the operands of the next stage overwrite the shared tiles
    }
    if (!ok) {
        if (status) atomicMax(status, PBR_ERR_CUDA);
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
