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
// The diabatic potential on tensor cores (pimc.py:1145-1150: the quadratic 'acef,debc,abdf->afbc'
// einsum, the linear einsum and the energies) as one GEMM with an extended K dimension:
//   V[row][pr] = sum_k a[row][k] * Bm[pr][k],   row = sample * P + bead, pr = pair_index(b, c).
// K is laid out in quads of four columns (d, e0 .. e0+3): a = s_d * s_e over the bead row's
// slots s = [q_0 .. q_{N-1}, 0 .. (to NA = N rounded up to 4), 1, 0, 0, 0].  Quads (d, e0) for
// d < N and e0 = 0, 4, .. <= d cover the quadratic pairs e <= d (Bm = the symmetrised 1/2 Q
// couplings, zero for e > d), quads (NA, j0) the linear terms (Bm = L_e for e < N), quad (NA, NA)
// the energies (Bm = E at its first column); quads (NA + 1, NA) = 0 pad K to a multiple of 32.
//
// TF32 with a hi/lo split of both operands: three MMAs per K step (hi*hi + hi*lo + lo*hi), FP32
// accumulation in TMEM, about 21 bits kept per product (the accuracy of the FP32 FMA form).
// Warp-specialised persistent CTA, one 128-row tile at a time:
//   warps 0-7   generate the A operand stage by stage (two threads per row, four quads each: one
//               broadcast load of q_d, one 128-bit load of q_e0..e0+3, hi / lo by masking to TF32)
//               from the tile's bead coordinates, which they prefetch one tile ahead (cp.async);
//   warp 8      issues the tcgen05.mma of each stage once its A and B operands are in place;
//   warp 9      streams the B stages (packed on the device in the shared-memory core layout) with
//               cp.async.bulk; when all stages fit they are loaded once and stay resident;
//   warps 10-13 read the finished accumulator out of TMEM and store V while the next tile runs.
// Stage buffers are handed over with mbarriers (full: producers arrived / bytes landed; empty:
// tcgen05.commit after the MMAs that read them); two TMEM accumulators let the MMAs of one tile
// run while the previous tile is read out.  Every wait is bounded: on a timeout a CTA records
// PBR_ERR_CUDA, every role leaves its loop, and the TMEM is freed after a bounded drain.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int kGenThreads = 256;                      // warps 0-7
constexpr int kEpiThreads = 128;                      // warps 10-13
constexpr int kPotThreads = kGenThreads + 64 + kEpiThreads;   // + MMA warp, B-loader warp, epilogue
constexpr int kQStageK = 32;                          // TF32 elements of K per stage (128 B)
constexpr int kQuadsPerStage = kQStageK / 4;
constexpr int kAStageCols = 2 * kQStageK;             // TMEM columns of one A stage (hi, lo)

// slot of the constant 1, and the number of slots per bead row (q, zeros, 1, 0, 0, 0)
__host__ __device__ inline int q_one(int N) { return (N + 3) / 4 * 4; }
__host__ __device__ inline int q_slots(int N) { return q_one(N) + 4; }

// number of quads before padding, and quad qi -> (d, e0)
__host__ __device__ inline int quad_count(int N) {
    int n = 0;
    for (int d = 0; d < N; ++d) n += (d + 4) / 4;
    return n + (N + 3) / 4 + 1;
}
__host__ __device__ inline void quad_of(int qi, int N, int& d, int& e0) {
    for (int dd = 0; dd < N; ++dd) {
        const int n = (dd + 4) / 4;
        if (qi < n) { d = dd; e0 = 4 * qi; return; }
        qi -= n;
    }
    const int nl = (N + 3) / 4, na = q_one(N);
    if (qi < nl) { d = na; e0 = 4 * qi; return; }       // linear
    if (qi == nl) { d = na; e0 = na; return; }          // energies
    d = na + 1; e0 = na;                                // padding: 0 * [1, 0, 0, 0]
}

// shared memory: B stages, two tiles of bead coordinates (mode-major: slot j of row r at
// j * 128 + r, so consecutive rows read consecutive words), the quad table, barriers.  The A
// operand never goes through shared memory: the generators store it into TMEM.
struct PotSmem {
    int nb, b, q, quads, bars, total;
    __host__ __device__ PotSmem(int N, int A2P, int nst, int nbuf) {
        nb = nbuf;
        int o = 0;
        b = o;     o += nb * 2 * A2P * kStageBytesK;                // [buffer][hi, lo]
        q = o;     o += 2 * kBM * q_slots(N) * 4;                   // two tiles
        quads = o; o += ((nst * kQuadsPerStage * 4 + 15) / 16) * 16;
        bars = o;  o += (3 * nb + 6) * 8 + 16;                      // barriers, TMEM slot, error flag
        total = o;
    }
};

// TMEM columns: two accumulators (2 x A2P), then nb A stages of 64 columns (hi 32, lo 32)
__host__ __device__ inline int pot_tmem_cols(int A2P, int nb) {
    int c = 32;
    while (c < 2 * A2P + nb * kAStageCols) c <<= 1;
    return c;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}\n"
                 ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// 16 consecutive FP32 accumulator columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_trunc(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
          "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
          "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
          "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
          "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
          "r"(__float_as_uint(v[15]))
        : "memory");
}

// D (TMEM) += A (TMEM, K-major: lane = row, 32-bit column = k) x B (shared memory descriptor)
__device__ __forceinline__ void mma_tf32_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n"
        ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// bounded wait that gives up early once another role has recorded an error
__device__ __forceinline__ bool mbar_wait_or_err(uint64_t* bar, uint32_t parity, volatile int* err) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
        if ((it & 1023u) == 1023u && *err) return false;
    }
    *err = 1;
    return false;
}

__global__ void __launch_bounds__(kPotThreads, 1) tc_potential_kernel(
        const float* __restrict__ q, int64_t X, int N, int P, int nst, int A2P, int nbuf,
        const unsigned char* __restrict__ bpack, float* __restrict__ vq, int ncols, int32_t* status) {
    extern __shared__ __align__(1024) unsigned char tsm[];
    const PotSmem L(N, A2P, nst, nbuf);
    const int NB = L.nb;
    unsigned char* sb = tsm + L.b;
    float* sq = reinterpret_cast<float*>(tsm + L.q);
    uint32_t* squad = reinterpret_cast<uint32_t*>(tsm + L.quads);
    uint64_t* full_a = reinterpret_cast<uint64_t*>(tsm + L.bars);
    uint64_t* full_b = full_a + NB;
    uint64_t* empty = full_b + NB;
    uint64_t* acc_full = empty + NB;
    uint64_t* acc_empty = acc_full + 2;
    uint64_t* sq_ready = acc_empty + 2;
    uint64_t* sq_done = sq_ready + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sq_done + 1);
    volatile int* err = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int NSL = q_slots(N);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t BSTAGE = static_cast<uint32_t>(A2P) * kStageBytesK;
    const int64_t rows = X * P;
    const int64_t tiles = (rows + kBM - 1) / kBM;
    const int my_tiles = static_cast<int>(tiles > blockIdx.x ? (tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0);
    const bool resident = nst <= NB;

    if (warp == 8) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < NB; ++i) {
            mbar_init(full_a + i, kGenThreads);
            mbar_init(full_b + i, 1);
            mbar_init(empty + i, 1);
        }
        for (int i = 0; i < 2; ++i) { mbar_init(acc_full + i, 1); mbar_init(acc_empty + i, kEpiThreads); }
        mbar_init(sq_ready, kGenThreads);
        mbar_init(sq_done, kGenThreads);
        *err = 0;
    }
    for (int i = tid; i < 2 * kBM * (NSL - N); i += kPotThreads) {     // the constant slots of both tiles
        const int t = i / (kBM * (NSL - N)), rem = i - t * kBM * (NSL - N);
        const int j = N + rem / kBM, r2 = rem % kBM;
        sq[t * kBM * NSL + j * kBM + r2] = (j == q_one(N)) ? 1.f : 0.f;
    }
    for (int qi = tid; qi < nst * kQuadsPerStage; qi += kPotThreads) {
        int d, e0;
        quad_of(qi, N, d, e0);
        squad[qi] = static_cast<uint32_t>(d) | (static_cast<uint32_t>(e0) << 16);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *tmem_slot;

    if (warp < 8) {
        // ======================= A-operand generators ==========================================
        // No named barriers here: every hand-over is an mbarrier with a bounded wait, and each
        // warp leaves the tile loop as a whole (warp-uniform ok), so a timeout cannot strand a
        // thread at a barrier that the others will never reach.
        const int row_l = tid & (kBM - 1), half = tid >> 7;
        const uint32_t lane_base = static_cast<uint32_t>((warp & 3) * 32) << 16;   // this warp's TMEM lanes
        // a tile's bead coordinates, copied asynchronously (4-byte cp.async straight into the
        // mode-major slots of buffer tl & 1) one tile ahead of their use; rows past the end are 0
        auto prefetch = [&](int tl) {
            float* dst = sq + (tl & 1) * kBM * NSL;
            const int64_t r0 = (static_cast<int64_t>(blockIdx.x) + static_cast<int64_t>(tl) * gridDim.x) * kBM;
            for (int i = tid; i < kBM * N; i += kGenThreads) {
                const int r2 = i % kBM, j = i / kBM;
                const int64_t row = r0 + r2;
                float* d = dst + j * kBM + r2;
                if (row < rows) {
                    const int64_t x = row / P;
                    const int p = static_cast<int>(row - x * P);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;"
                                 ::"r"(smem_u32(d)), "l"(q + (x * N + j) * P + p) : "memory");
                } else {
                    *d = 0.f;
                }
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        };
        int it = 0;
        bool ok = true;
        if (my_tiles > 0) prefetch(0);
        for (int tl = 0; tl < my_tiles; ++tl) {
            ok = __all_sync(0xffffffffu, ok && !*err);
            if (!ok) break;
            // buffer (tl + 1) & 1 is free once every generator has finished tile tl - 1
            if (tl > 0) ok = mbar_wait_or_err(sq_done, (tl - 1) & 1, err);
            const bool ahead = ok && tl + 1 < my_tiles;
            if (ahead) prefetch(tl + 1);
            if (ok) {
                if (ahead) asm volatile("cp.async.wait_group 1;" ::: "memory");
                else asm volatile("cp.async.wait_group 0;" ::: "memory");
                mbar_arrive(sq_ready);
                ok = mbar_wait_or_err(sq_ready, tl & 1, err);
            }
            const float* myq = sq + (tl & 1) * kBM * NSL + row_l;
            for (int st = 0; st < nst; ++st, ++it) {
                const int b = it % NB, use = it / NB;
                if (ok && use > 0) ok = mbar_wait_or_err(empty + b, (use - 1) & 1, err);
                if (!ok) continue;
                // this thread's row, K columns half * 16 .. half * 16 + 15 of the stage
                float hi[16], lo[16];
#pragma unroll
                for (int u = 0; u < kQuadsPerStage / 2; ++u) {
                    const uint32_t de = squad[st * kQuadsPerStage + half * (kQuadsPerStage / 2) + u];
                    const int d = static_cast<int>(de & 0xFFFFu), e0 = static_cast<int>(de >> 16);
                    const float qd = myq[d * kBM];
#pragma unroll
                    for (int v = 0; v < 4; ++v) {
                        const float x = qd * myq[(e0 + v) * kBM];
                        const float h = tf32_trunc(x);
                        hi[4 * u + v] = h;
                        lo[4 * u + v] = x - h;           // the tensor core reads its TF32 bits
                    }
                }
                const uint32_t col = static_cast<uint32_t>(2 * A2P + b * kAStageCols + half * 16);
                tmem_st16(tmem + lane_base + col, hi);
                tmem_st16(tmem + lane_base + col + kQStageK, lo);
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                mbar_arrive(full_a + b);
            }
            if (ok) mbar_arrive(sq_done);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");          // no copy in flight at exit
    } else if (warp >= 10) {
        // ======================= epilogue warpgroup: TMEM -> V =================================
        const int lg = warp & 3;                                  // TMEM lanes 32 lg .. 32 lg + 31
        bool ok = true;
        for (int tl = 0; tl < my_tiles; ++tl) {
            ok = __all_sync(0xffffffffu, ok && !*err);
            if (!ok) break;
            const int acc = tl & 1;
            ok = mbar_wait_or_err(acc_full + acc, (tl >> 1) & 1, err);
            ok = __all_sync(0xffffffffu, ok);                     // tcgen05.ld is warp-collective
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const int64_t r0 = (static_cast<int64_t>(blockIdx.x) + static_cast<int64_t>(tl) * gridDim.x) * kBM;
            const int64_t row = r0 + lg * 32 + lane;
            for (int c0 = 0; c0 < A2P; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + (static_cast<uint32_t>(lg * 32) << 16) + static_cast<uint32_t>(acc * A2P + c0), v);
                if (row < rows) {
                    float* dst = vq + row * A2P + c0;
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(acc_empty + acc);
        }
    } else if (warp == 8) {
        // ======================= MMA issuer (one thread) =======================================
        if (lane == 0) {
            const uint32_t idesc = instr_desc(2, kBM, A2P);
            constexpr uint32_t LBO = 128, SBO = (kStageBytesK / 16) * 128;
            uint64_t* last = nullptr;                 // barrier and parity of the latest commit
            uint32_t lastp = 0;
            int it = 0;
            for (int tl = 0; tl < my_tiles && !*err; ++tl) {
                const int acc = tl & 1;
                if (tl >= 2 && !mbar_wait_or_err(acc_empty + acc, ((tl >> 1) - 1) & 1, err)) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const uint32_t dtm = tmem + static_cast<uint32_t>(acc * A2P);
                bool ok = true;
                for (int st = 0; st < nst; ++st, ++it) {
                    const int b = it % NB, use = it / NB;
                    if (!mbar_wait_or_err(full_a + b, use & 1, err) ||
                        !mbar_wait_or_err(full_b + (resident ? st : b), resident ? 0u : (use & 1), err)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const uint32_t ahi = tmem + static_cast<uint32_t>(2 * A2P + b * kAStageCols);
                    const uint32_t alo = ahi + kQStageK;
                    const unsigned char* bhi = sb + (resident ? st : b) * 2 * BSTAGE;
                    const unsigned char* blo = bhi + BSTAGE;
#pragma unroll
                    for (int kk = 0; kk < kQStageK; kk += 8) {
                        const uint32_t off = static_cast<uint32_t>(kk * 4 / 16) * 128;
                        const uint64_t dbh = smem_desc(smem_u32(bhi) + off, LBO, SBO);
                        const uint64_t dbl = smem_desc(smem_u32(blo) + off, LBO, SBO);
                        mma_tf32_ts(dtm, ahi + kk, dbh, idesc, (st > 0 || kk > 0) ? 1u : 0u);
                        mma_tf32_ts(dtm, ahi + kk, dbl, idesc, 1u);
                        mma_tf32_ts(dtm, alo + kk, dbh, idesc, 1u);
                    }
                    mma_commit(empty + b);
                    last = empty + b;
                    lastp = use & 1;
                }
                if (!ok) break;
                mma_commit(acc_full + acc);
                last = acc_full + acc;
                lastp = (tl >> 1) & 1;
            }
            if (*err && last) mbar_wait(last, lastp);          // bounded drain of the MMAs in flight
        }
    } else {
        // ======================= B-stage loader (one thread) ===================================
        if (lane == 0) {
            if (resident) {
                for (int st = 0; st < nst && my_tiles > 0; ++st) {
                    mbar_expect_tx(full_b + st, 2 * BSTAGE);
                    bulk_g2s(sb + st * 2 * BSTAGE, bpack + static_cast<int64_t>(st) * 2 * BSTAGE, 2 * BSTAGE,
                             full_b + st);
                }
                if (*err)
                    for (int st = 0; st < nst && my_tiles > 0; ++st) mbar_wait(full_b + st, 0);   // bounded drain
            } else {
                const int total = my_tiles * nst;
                uint64_t* last = nullptr;
                uint32_t lastp = 0;
                for (int it = 0; it < total && !*err; ++it) {
                    const int b = it % NB, use = it / NB, st = it % nst;
                    if (use > 0 && !mbar_wait_or_err(empty + b, (use - 1) & 1, err)) break;
                    mbar_expect_tx(full_b + b, 2 * BSTAGE);
                    bulk_g2s(sb + b * 2 * BSTAGE, bpack + static_cast<int64_t>(st) * 2 * BSTAGE, 2 * BSTAGE,
                             full_b + b);
                    last = full_b + b;
                    lastp = use & 1;
                }
                if (*err && last) mbar_wait(last, lastp);      // bounded drain of the copy in flight
            }
        }
    }
    __syncthreads();
    if (*err && tid == 0 && status) atomicMax(status, PBR_ERR_CUDA);
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 8)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Qp [N2][A2], L [N][A2], E [A2] (FP32 or FP64; L and E nullable = zero) -> TF32 hi / lo in the
// stage-major shared-memory core layout: stage s = [hi: A2P rows][lo: A2P rows], each row's 32
// K columns as 8 cores of 4, core (row r, column c) at ((r / 8) * 8 + c) * 8 + r % 8 (16 B units).
template <typename T>
__global__ void tc_pack_kernel(const T* __restrict__ qq, const T* __restrict__ lin, const T* __restrict__ en, int N,
                               int A2, int nst, int A2P, float* __restrict__ out) {
    const int64_t n = static_cast<int64_t>(nst) * A2P * kQStageK;      // (stage, row, k in stage)
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int st = static_cast<int>(i / (static_cast<int64_t>(A2P) * kQStageK));
        const int rem = static_cast<int>(i - static_cast<int64_t>(st) * A2P * kQStageK);
        const int pr = rem / kQStageK, kk = rem - pr * kQStageK;
        const int qi = st * kQuadsPerStage + kk / 4, u = kk % 4;
        int d, e0;
        quad_of(qi, N, d, e0);
        const int e = e0 + u;
        float x = 0.f;
        const int na = q_one(N);
        if (pr < A2) {
            if (d < N) {
                if (e <= d) x = static_cast<float>(qq[static_cast<int64_t>(d * (d + 1) / 2 + e) * A2 + pr]);
            } else if (d == na && e0 < N) {
                if (e < N && lin) x = static_cast<float>(lin[static_cast<int64_t>(e) * A2 + pr]);
            } else if (d == na && e0 == na) {
                if (u == 0 && en) x = static_cast<float>(en[pr]);
            }
        }
        const float h = tf32_rna(x);
        const int c = kk / 4;
        const int64_t base = static_cast<int64_t>(st) * 2 * A2P * kQStageK;
        const int64_t slot = (static_cast<int64_t>((pr >> 3) * (kStageBytesK / 16) + c) * 8 + (pr & 7)) * 4 + u;
        out[base + slot] = h;
        out[base + static_cast<int64_t>(A2P) * kQStageK + slot] = tf32_rna(x - h);
    }
}

// stage buffers: as many as 4 that fit both the shared memory (B stages) and the TMEM (A stages
// beside the two accumulators)
int pot_buffers(int N, int A2P, int nst) {
    for (int nb = 4; nb >= 2; --nb)
        if (PotSmem(N, A2P, nst, nb).total <= 227 * 1024 && 2 * A2P + nb * kAStageCols <= 512) return nb;
    return 0;
}

}  // namespace

namespace pbr {

int tc_quadratic_cols(int A) { return (A * (A + 1) / 2 + 15) / 16 * 16; }
int tc_quadratic_kdim(int N) { return (quad_count(N) + kQuadsPerStage - 1) / kQuadsPerStage * kQStageK; }
int64_t tc_packed_floats(int N, int A) { return static_cast<int64_t>(2) * tc_quadratic_cols(A) * tc_quadratic_kdim(N); }

int tc_quadratic_launch(const float* q, int64_t X, int N, int P, int A2P, const void* bpack, float* vq,
                        int32_t* status, cudaStream_t stream) {
    if (!q || !bpack || !vq || X < 0 || N < 1 || N > 64 || P < 1) return PBR_ERR_ARG;
    if (A2P < 16 || A2P > 144 || A2P % 16 != 0) return PBR_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(bpack) | reinterpret_cast<uintptr_t>(vq)) & 15) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const int nst = tc_quadratic_kdim(N) / kQStageK;
    const int nb = pot_buffers(N, A2P, nst);
    if (nb == 0) return PBR_ERR_UNSUPPORTED;
    const int ncols = pot_tmem_cols(A2P, nb);
    const PotSmem L(N, A2P, nst, nb);
    static int configured = 0;
    if (L.total > configured) {
        if (cudaFuncSetAttribute(tc_potential_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = 227 * 1024;
    }
    int dev = 0, sms = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t tiles = (X * P + kBM - 1) / kBM;
    // one CTA per SM: at least half the shared memory each, so two CTAs never share an SM's TMEM
    const int smem = L.total > 116 * 1024 ? L.total : 116 * 1024;
    const int grid = static_cast<int>(tiles < sms ? tiles : sms);
    tc_potential_kernel<<<grid, kPotThreads, smem, stream>>>(q, X, N, P, nst, A2P, nb,
                                                                 static_cast<const unsigned char*>(bpack), vq,
                                                                 ncols, status);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int tc_pack_launch(const void* qq, const void* lin, const void* en, int precision, int N, int A, void* bpack,
                   cudaStream_t stream) {
    if (!qq || !bpack || N < 1 || N > 64 || A < 1 || A > 16) return PBR_ERR_ARG;
    const int A2 = A * (A + 1) / 2;
    const int nst = tc_quadratic_kdim(N) / kQStageK, A2P = tc_quadratic_cols(A);
    const int64_t n = static_cast<int64_t>(nst) * A2P * kQStageK;
    const int grid = static_cast<int>((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    float* out = static_cast<float*>(bpack);
    if (precision == 32)
        tc_pack_kernel<float><<<grid, 256, 0, stream>>>(static_cast<const float*>(qq), static_cast<const float*>(lin),
                                                        static_cast<const float*>(en), N, A2, nst, A2P, out);
    else if (precision == 64)
        tc_pack_kernel<double><<<grid, 256, 0, stream>>>(static_cast<const double*>(qq), static_cast<const double*>(lin),
                                                         static_cast<const double*>(en), N, A2, nst, A2P, out);
    else
        return PBR_ERR_ARG;
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

}  // namespace pbr

extern "C" {

int pbr_tc_potential_dims(int32_t N, int32_t A, int32_t* n2p, int32_t* a2p) {
    if (N < 1 || N > 64 || A < 1 || A > 16 || !n2p || !a2p) return PBR_ERR_ARG;
    *n2p = pbr::tc_quadratic_kdim(N);
    *a2p = pbr::tc_quadratic_cols(A);
    return PBR_OK;
}

int64_t pbr_tc_potential_packed_floats(int32_t N, int32_t A) {
    if (N < 1 || N > 64 || A < 1 || A > 16) return -1;
    return pbr::tc_packed_floats(N, A);
}

int pbr_tc_pack_potential(const void* vib_qq, const void* vib_l, const void* vib_e, int32_t precision, int32_t N,
                          int32_t A, void* b_packed, void* stream) {
    return pbr::tc_pack_launch(vib_qq, vib_l, vib_e, precision, N, A, b_packed, static_cast<cudaStream_t>(stream));
}

int pbr_tc_potential(const float* q, int64_t X, int32_t N, int32_t P, int32_t A, const void* b_packed, float* vq,
                     int32_t* status, void* stream) {
    if (A < 1 || A > 16) return PBR_ERR_ARG;
    return pbr::tc_quadratic_launch(q, X, N, P, pbr::tc_quadratic_cols(A), b_packed, vq, status,
                                    static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Tensor-pipe rate probe: each CTA (one per SM) issues `reps` back-to-back tcgen05.mma kind::tf32
// (M x N x 8, operands zeros in shared memory, one TMEM accumulator) from one thread, commits once
// and waits (bounded).  Reports the issuing thread's cycles per MMA and the whole-GPU TF/s; the
// denominator the potential GEMM is held against.
// ---------------------------------------------------------------------------------------------
namespace {

__global__ void tc_rate_kernel(int M, int N, int reps, int32_t* flag, long long* cycles) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* sa = sm;                 // 128 rows x 32 B (K = 8 tf32)
    unsigned char* sb = sm + 128 * 32;      // 256 rows x 32 B
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 128 * 32 + 256 * 32);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    for (int i = threadIdx.x; i < (128 + 256) * 32 / 4; i += blockDim.x) reinterpret_cast<float*>(sm)[i] = 0.f;
    int ncols = 32;
    while (ncols < N) ncols <<= 1;
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) mbar_init(bar, 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = *slot;
    if (threadIdx.x == 0) {
        const uint32_t idesc = instr_desc(2, M, N);
        const uint64_t da = smem_desc(smem_u32(sa), 128, 256), db = smem_desc(smem_u32(sb), 128, 256);
        const long long t0 = clock64();
        for (int i = 0; i < reps; ++i) mma_issue<2>(tmem, da, db, idesc, i > 0 ? 1u : 0u);
        mma_commit(bar);
        const bool done = mbar_wait(bar, 0);
        const long long t1 = clock64();
        if (!done) atomicExch(flag, 1);
        if (blockIdx.x == 0) *cycles = t1 - t0;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

}  // namespace

extern "C" int pbr_tc_mma_rate(int32_t M, int32_t N, int32_t reps, void* scratch, double* tflops,
                               double* cycles_per_mma, void* stream) {
    if ((M != 64 && M != 128) || N < 16 || N > 256 || N % 16 != 0 || reps < 1 || reps > (1 << 20) || !tflops ||
        !cycles_per_mma || !scratch || (reinterpret_cast<uintptr_t>(scratch) & 7) != 0)
        return PBR_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    constexpr int kSmem = 120 * 1024;      // one CTA per SM
    if (cudaFuncSetAttribute(tc_rate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem) != cudaSuccess)
        return PBR_ERR_UNSUPPORTED;
    // the caller's 16 bytes: the cycle count (8-byte aligned) and the bounded-wait flag after it
    long long* dcyc = static_cast<long long*>(scratch);
    int32_t* dflag = reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + 8);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = PBR_OK;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = PBR_ERR_CUDA;
    if (rc == PBR_OK && cudaMemsetAsync(scratch, 0, 16, st) != cudaSuccess) rc = PBR_ERR_CUDA;
    if (rc == PBR_OK) {
        tc_rate_kernel<<<sms, 128, kSmem, st>>>(M, N, 64, dflag, dcyc);        // warm-up
        cudaEventRecord(e0, st);
        tc_rate_kernel<<<sms, 128, kSmem, st>>>(M, N, reps, dflag, dcyc);
        cudaEventRecord(e1, st);
        if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) rc = PBR_ERR_CUDA;
    }
    float ms = 0.f;
    long long cyc = 0;
    int32_t flag = 0;
    if (rc == PBR_OK && (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
                         cudaMemcpyAsync(&cyc, dcyc, sizeof(cyc), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                         cudaMemcpyAsync(&flag, dflag, sizeof(flag), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                         cudaStreamSynchronize(st) != cudaSuccess))
        rc = PBR_ERR_CUDA;
    if (rc == PBR_OK && flag) rc = PBR_ERR_CUDA;      // a wait in the kernel gave up
    *tflops = (rc == PBR_OK && ms > 0.f) ? 2.0 * M * N * 8.0 * reps * sms / (ms * 1e-3) / 1e12 : 0.0;
    *cycles_per_mma = rc == PBR_OK ? static_cast<double>(cyc) / reps : 0.0;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}
