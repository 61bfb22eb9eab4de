// pbr_tc.cu -- 5th-generation tensor-core (tcgen05) GEMM for sm_103a, written with inline PTX:
// operands staged in shared memory in the canonical no-swizzle K-major layout, one elected thread
// issues tcgen05.mma into a TMEM accumulator, completion is signalled through an mbarrier
// (tcgen05.commit), and the warps read the accumulator back with tcgen05.ld.
//
// pbr_tc_gemm: C[M][N] (FP32) = A[M][K] * B[N][K]^T for BF16 or TF32 operands, M % 128 == 0,
// N % 16 == 0 (16 <= N <= 256), K a multiple of the stage depth.  Every wait is bounded: on a
// timeout the CTA records PBR_ERR_CUDA in *status, skips the rest of its work, and still frees
// its TMEM.
#include <algorithm>
#include <cstdint>

#include <cuda_fp16.h>

#include "pbr_common.cuh"
#include "pbr_tcgen05.cuh"

namespace {

constexpr int kTcThreads = 128;          // one warpgroup: warp w reads TMEM lanes 32w .. 32w+31
constexpr int kBM = 128;
constexpr int kStageBytesK = 128;        // bytes of K per stage (64 bf16 or 32 tf32)
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
// the energies (Bm = E at its first column); quads (NA + 1, NA) = 0 pad K to a multiple of 64.
//
// FP16 with a hi/lo split of both operands: three tcgen05.mma kind::f16 per K step of 16
// (hi*hi + hi*lo + lo*hi), FP32 accumulation in TMEM, about 22 bits kept per product (the
// accuracy of the FP32 FMA form).  A kind::f16 MMA of M = 128, K = 16 costs 74 cycles for any
// N <= 128 on GB300, a kind::tf32 one of K = 8 costs 142 (measured by pbr_tc_mma_rate), so the
// FP16 split does the same K in 26 % of the tensor-pipe time of a TF32 split.  FP16's range is
// kept by exact power-of-two scaling: every bead row's products are scaled by 2^s_row so that
// the largest is below 2^14 (its largest coordinate squared decides s_row), the couplings by one
// global 2^s_B so that the largest is below 2^14; hi and lo then stay normal FP16 numbers except
// for entries 2^-25 or less of the largest, whose absolute error is below 2^-39 of it.  The
// first padding column of the couplings (pair A2, always < A2P for A <= 16) holds 1 at the
// energies' K column, so the accumulator's column A2 returns 2^s_row for its row, and the
// epilogue divides the row by 2^s_row * 2^s_B exactly.
// Warp-specialised persistent CTA, one 128-row tile at a time:
//   warps 0-7   generate the A operand stage by stage (two threads per row, eight quads each: the
//               row's q_d and q_e0..e0+3 from shared memory, hi / lo as FP16 pairs) from the
//               tile's bead coordinates, which they prefetch one tile ahead (cp.async);
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
constexpr int kQStageK = 64;                          // FP16 elements of K per stage (128 B per row)
constexpr int kQuadsPerStage = kQStageK / 4;
constexpr int kAPartCols = kQStageK / 2;              // TMEM columns of one A part (two FP16 per column)
constexpr int kAStageCols = 2 * kAPartCols;           // TMEM columns of one A stage (hi, lo)
constexpr int kKMma = 16;                             // K of one kind::f16 MMA

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

// K column of the energies (the first column of quad (NA, NA)), where a = 1 for every row
__host__ __device__ inline int energy_column(int N) { return 4 * (quad_count(N) - 1); }

// power of two 2^(14 - e) with x < 2^e (x positive, normal, finite): x * result < 2^14
__device__ __forceinline__ float fp16_range_scale(float x) {
    const int e = static_cast<int>((__float_as_uint(x) >> 23) & 0xFFu) - 126;
    return __uint_as_float(static_cast<uint32_t>(127 + 14 - e) << 23);
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

// one FP32 accumulator column of this warp's 32 TMEM lanes
__device__ __forceinline__ float tmem_ld1(uint32_t taddr) {
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    return __uint_as_float(r);
}

// 16 consecutive 32-bit TMEM columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]),
          "r"(v[8]), "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16]) {
    uint32_t u[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) u[i] = __float_as_uint(v[i]);
    tmem_st16(taddr, u);
}

// D (TMEM) += A (TMEM, K-major: lane = row, 32-bit column = k) x B (shared memory descriptor)
__device__ __forceinline__ void mma_tf32_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n"
        ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// D (TMEM) += A (TMEM, K-major: lane = row, 32-bit column = the FP16 pair k, k + 1 with k in the
// low half) x B (shared memory descriptor, FP16); both operands FP16
__device__ __forceinline__ void mma_f16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t idesc,
                                           uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n}\n"
        ::"r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

using pbr::pack_f16x2;
using pbr::split_f16x2;

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
        const float* __restrict__ q, int64_t X, int N, int P, int nst, int A2, int A2P, int nbuf,
        const unsigned char* __restrict__ bpack, const float* __restrict__ b_scale, float* __restrict__ vq,
        int ncols, int32_t* status) {
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
            // the row's scale 2^s_row: its largest product (max(1, max_j q_j^2)) times 2^s_row
            // stays below 2^14; NaN or Inf coordinates leave the products non-finite
            float qmax = 1.f;
            for (int j = 0; j < N; ++j) qmax = fmaxf(qmax, fabsf(myq[j * kBM]));
            const float srow = fp16_range_scale(fminf(qmax * qmax, 3.0e38f));
            for (int st = 0; st < nst; ++st, ++it) {
                const int b = it % NB, use = it / NB;
                if (ok && use > 0) ok = mbar_wait_or_err(empty + b, (use - 1) & 1, err);
                if (!ok) continue;
                // this thread's row, K columns half * 32 .. half * 32 + 31 of the stage
                uint32_t hi[16], lo[16];
#pragma unroll
                for (int u = 0; u < kQuadsPerStage / 2; ++u) {
                    const uint32_t de = squad[st * kQuadsPerStage + half * (kQuadsPerStage / 2) + u];
                    const int d = static_cast<int>(de & 0xFFFFu), e0 = static_cast<int>(de >> 16);
                    const float qd = myq[d * kBM] * srow;
                    const float x0 = qd * myq[e0 * kBM], x1 = qd * myq[(e0 + 1) * kBM];
                    const float x2 = qd * myq[(e0 + 2) * kBM], x3 = qd * myq[(e0 + 3) * kBM];
                    split_f16x2(x0, x1, hi[2 * u], lo[2 * u]);
                    split_f16x2(x2, x3, hi[2 * u + 1], lo[2 * u + 1]);
                }
                const uint32_t col = static_cast<uint32_t>(2 * A2P + b * kAStageCols + half * 16);
                tmem_st16(tmem + lane_base + col, hi);
                tmem_st16(tmem + lane_base + col + kAPartCols, lo);
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
        const float sb_inv = 1.0f / *b_scale;                     // 2^-s_B
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
            const uint32_t tbase = tmem + (static_cast<uint32_t>(lg * 32) << 16) + static_cast<uint32_t>(acc * A2P);
            // column A2 = 2^s_row exactly: V = D / (2^s_row 2^s_B), exact powers of two
            const float inv = sb_inv / tmem_ld1(tbase + static_cast<uint32_t>(A2));
            for (int c0 = 0; c0 < A2P; c0 += 16) {
                float v[16];
                tmem_ld16(tbase + static_cast<uint32_t>(c0), v);
                if (row < rows) {
                    float* dst = vq + row * A2P + c0;
#pragma unroll
                    for (int i = 0; i < 16; i += 4)
                        *reinterpret_cast<float4*>(dst + i) =
                            make_float4(v[i] * inv, v[i + 1] * inv, v[i + 2] * inv, v[i + 3] * inv);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(acc_empty + acc);
        }
    } else if (warp == 8) {
        // ======================= MMA issuer (one thread) =======================================
        if (lane == 0) {
            const uint32_t idesc = instr_desc(0, kBM, A2P);        // FP16 x FP16 -> FP32
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
                    const uint32_t alo = ahi + kAPartCols;
                    const unsigned char* bhi = sb + (resident ? st : b) * 2 * BSTAGE;
                    const unsigned char* blo = bhi + BSTAGE;
#pragma unroll
                    for (int kk = 0; kk < kQStageK; kk += kKMma) {
                        const uint32_t off = static_cast<uint32_t>(kk * 2 / 16) * 128;   // cores along K
                        const uint64_t dbh = smem_desc(smem_u32(bhi) + off, LBO, SBO);
                        const uint64_t dbl = smem_desc(smem_u32(blo) + off, LBO, SBO);
                        const uint32_t acol = static_cast<uint32_t>(kk / 2);            // two FP16 per column
                        mma_f16_ts(dtm, ahi + acol, dbh, idesc, (st > 0 || kk > 0) ? 1u : 0u);
                        mma_f16_ts(dtm, ahi + acol, dbl, idesc, 1u);
                        mma_f16_ts(dtm, alo + acol, dbh, idesc, 1u);
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

// The largest |entry| of Qp [N2][A2], L [N][A2], E [A2] (L, E nullable) into *maxbits (the bits
// of a non-negative float, which order like the floats; zeroed by the caller): a grid-stride
// maximum per block, then one atomicMax per block.
template <typename T>
__global__ void tc_pack_max_kernel(const T* __restrict__ qq, const T* __restrict__ lin, const T* __restrict__ en,
                                   int N, int A2, unsigned int* __restrict__ maxbits) {
    __shared__ float red[32];
    const int64_t nq = static_cast<int64_t>(N) * (N + 1) / 2 * A2, nl = lin ? static_cast<int64_t>(N) * A2 : 0,
                  ne = en ? A2 : 0;
    float m = 0.f;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < nq + nl + ne;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const T x = i < nq ? qq[i] : (i < nq + nl ? lin[i - nq] : en[i - nq - nl]);
        m = fmaxf(m, fminf(fabsf(static_cast<float>(x)), 3.0e38f));
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < static_cast<int>(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
        atomicMax(maxbits, __float_as_uint(m));
    }
}

// 2^s_B from the largest |entry| m: m 2^s_B < 2^14 (1 when every entry is zero)
__device__ __forceinline__ float coupling_scale(unsigned int maxbits) {
    const float m = __uint_as_float(maxbits);
    return m > 0.f ? fp16_range_scale(fmaxf(m, 1.0e-30f)) : 1.f;
}

// Qp [N2][A2], L [N][A2], E [A2] (FP32 or FP64; L and E nullable = zero), times 2^s_B -> FP16
// hi / lo in the stage-major shared-memory core layout: stage s = [hi: A2P rows][lo: A2P rows],
// each row's 64 K columns as 8 cores of 8, core (row r, column c) at ((r / 8) * 8 + c) * 8 + r % 8
// (16 B units), column k of the core in half k % 8.  Row A2 holds 1 at the energies' K column.
// tail[0] holds the largest |entry| (tc_pack_max_kernel); block 0 writes 2^s_B to tail[1].
template <typename T>
__global__ void tc_pack_kernel(const T* __restrict__ qq, const T* __restrict__ lin, const T* __restrict__ en, int N,
                               int A2, int nst, int A2P, unsigned int* __restrict__ tail, __half* __restrict__ out) {
    const int64_t n = static_cast<int64_t>(nst) * A2P * kQStageK;      // (stage, row, k in stage)
    const float sB = coupling_scale(tail[0]);
    if (blockIdx.x == 0 && threadIdx.x == 0) reinterpret_cast<float*>(tail)[1] = sB;
    const int kone = energy_column(N);
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
            x *= sB;
        } else if (pr == A2 && st * kQStageK + kk == kone) {
            x = 1.f;
        }
        const __half h = __float2half_rn(x);
        const int c = kk / 8;
        const int64_t base = static_cast<int64_t>(st) * 2 * A2P * kQStageK;
        const int64_t slot = (static_cast<int64_t>((pr >> 3) * (kStageBytesK / 16) + c) * 8 + (pr & 7)) * 8 + kk % 8;
        out[base + slot] = h;
        out[base + static_cast<int64_t>(A2P) * kQStageK + slot] = __float2half_rn(x - __half2float(h));
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
// FP16 hi and lo of A2P x K couplings (one 32-bit word per two), then 4 words: the largest
// |coupling| and the scale 2^s_B
int64_t tc_packed_floats(int N, int A) {
    return static_cast<int64_t>(tc_quadratic_cols(A)) * tc_quadratic_kdim(N) + 4;
}

int tc_quadratic_launch(const float* q, int64_t X, int N, int P, int A, const void* bpack, float* vq,
                        int32_t* status, cudaStream_t stream) {
    if (!q || !bpack || !vq || X < 0 || N < 1 || N > 64 || P < 1 || A < 1 || A > 16) return PBR_ERR_ARG;
    const int A2 = A * (A + 1) / 2, A2P = tc_quadratic_cols(A);
    if (A2P > 144) return PBR_ERR_ARG;
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
    const auto* bp = static_cast<const unsigned char*>(bpack);
    const float* scale = reinterpret_cast<const float*>(bp + static_cast<int64_t>(A2P) * tc_quadratic_kdim(N) * 4) + 1;
    tc_potential_kernel<<<grid, kPotThreads, smem, stream>>>(q, X, N, P, nst, A2, A2P, nb, bp, scale, vq, ncols,
                                                                 status);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

int tc_pack_launch(const void* qq, const void* lin, const void* en, int precision, int N, int A, void* bpack,
                   cudaStream_t stream) {
    if (!qq || !bpack || N < 1 || N > 64 || A < 1 || A > 16) return PBR_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(bpack) & 15) return PBR_ERR_ARG;
    const int A2 = A * (A + 1) / 2;
    const int nst = tc_quadratic_kdim(N) / kQStageK, A2P = tc_quadratic_cols(A);
    const int64_t n = static_cast<int64_t>(nst) * A2P * kQStageK;
    const int grid = static_cast<int>((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    auto* out = static_cast<__half*>(bpack);
    // the two tail words after the 2 x A2P x K FP16 values (A2P x K x 4 bytes)
    auto* tail = reinterpret_cast<unsigned int*>(static_cast<unsigned char*>(bpack) + static_cast<int64_t>(A2P) * nst *
                                                 kQStageK * 4);
    const int64_t nin = static_cast<int64_t>(N) * (N + 1) / 2 * A2 + static_cast<int64_t>(N + 1) * A2;
    const int mgrid = static_cast<int>(std::min<int64_t>((nin + 255) / 256, 304));
    if (cudaMemsetAsync(tail, 0, sizeof(unsigned int), stream) != cudaSuccess) return PBR_ERR_CUDA;
    if (precision == 32) {
        tc_pack_max_kernel<float><<<mgrid, 256, 0, stream>>>(static_cast<const float*>(qq), static_cast<const float*>(lin),
                                                             static_cast<const float*>(en), N, A2, tail);
        tc_pack_kernel<float><<<grid, 256, 0, stream>>>(static_cast<const float*>(qq), static_cast<const float*>(lin),
                                                        static_cast<const float*>(en), N, A2, nst, A2P, tail, out);
    } else if (precision == 64) {
        tc_pack_max_kernel<double><<<mgrid, 256, 0, stream>>>(static_cast<const double*>(qq),
                                                              static_cast<const double*>(lin),
                                                              static_cast<const double*>(en), N, A2, tail);
        tc_pack_kernel<double><<<grid, 256, 0, stream>>>(static_cast<const double*>(qq), static_cast<const double*>(lin),
                                                         static_cast<const double*>(en), N, A2, nst, A2P, tail, out);
    } else {
        return PBR_ERR_ARG;
    }
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
    return pbr::tc_quadratic_launch(q, X, N, P, A, b_packed, vq, status, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Tensor-pipe rate probe: each CTA (one per SM) issues `reps` back-to-back tcgen05.mma (kind::tf32,
// M x N x 8, or kind::f16 with 16-bit operands, M x N x 16; operands zeros in shared memory, or the
// A operand in TMEM) from one thread, round-robin over nacc independent TMEM accumulators,
// commits once and waits (bounded).  Reports the issuing thread's cycles per MMA and the
// whole-GPU TF/s: the denominator the potential GEMM is held against, and the evidence for what
// an instruction costs (its shape, its operand type, its accumulator dependencies).
// ---------------------------------------------------------------------------------------------
namespace {

__global__ void tc_rate_kernel(int fmt, int M, int N, int nacc, int a_tmem, int reps, int32_t* flag,
                               long long* cycles) {
    extern __shared__ __align__(1024) unsigned char sm[];
    unsigned char* sa = sm;                 // 128 rows x 32 B (K = 8 tf32 or 16 bf16)
    unsigned char* sb = sm + 128 * 32;      // 256 rows x 32 B
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 128 * 32 + 256 * 32);
    uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
    for (int i = threadIdx.x; i < (128 + 256) * 32 / 4; i += blockDim.x) reinterpret_cast<float*>(sm)[i] = 0.f;
    int ncols = 32;
    while (ncols < nacc * N + (a_tmem ? 16 : 0)) ncols <<= 1;
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
    const uint32_t ta = tmem + static_cast<uint32_t>(nacc * N);      // A operand: 16 columns (TMEM form)
    if (a_tmem) {
        // zero this warp's lanes of the A columns (warps 0-3 cover the 128 lanes)
        float z[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) z[i] = 0.f;
        const uint32_t lanes = static_cast<uint32_t>((threadIdx.x >> 5) * 32) << 16;
        tmem_st16(ta + lanes, z);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (threadIdx.x == 0) {
        const uint32_t idesc = instr_desc(fmt, M, N);
        const uint64_t da = smem_desc(smem_u32(sa), 128, 256), db = smem_desc(smem_u32(sb), 128, 256);
        const long long t0 = clock64();
        int acc = 0;
        for (int i = 0; i < reps; ++i) {
            const uint32_t d = tmem + static_cast<uint32_t>(acc * N);
            const uint32_t accumulate = i >= nacc ? 1u : 0u;
            if (fmt == 1 && a_tmem) mma_f16_ts(d, ta, db, idesc, accumulate);
            else if (fmt == 1) mma_issue<1>(d, da, db, idesc, accumulate);
            else if (a_tmem) mma_tf32_ts(d, ta, db, idesc, accumulate);
            else mma_issue<2>(d, da, db, idesc, accumulate);
            if (++acc == nacc) acc = 0;
        }
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

extern "C" int pbr_tc_mma_rate(int32_t fmt, int32_t M, int32_t N, int32_t nacc, int32_t a_tmem, int32_t reps,
                               void* scratch, double* tflops, double* cycles_per_mma, void* stream) {
    if ((fmt != 1 && fmt != 2) || (M != 64 && M != 128) || N < 16 || N > 256 || N % 16 != 0 || nacc < 1 ||
        nacc > 4 || nacc * N + (a_tmem ? 16 : 0) > 512 || (a_tmem && M != 128) || reps < 1 ||
        reps > (1 << 20) || !tflops || !cycles_per_mma || !scratch || (reinterpret_cast<uintptr_t>(scratch) & 7) != 0)
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
        tc_rate_kernel<<<sms, 128, kSmem, st>>>(fmt, M, N, nacc, a_tmem, 64, dflag, dcyc);        // warm-up
        cudaEventRecord(e0, st);
        tc_rate_kernel<<<sms, 128, kSmem, st>>>(fmt, M, N, nacc, a_tmem, reps, dflag, dcyc);
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
    const double kdim = fmt == 1 ? 16.0 : 8.0;
    *tflops = (rc == PBR_OK && ms > 0.f) ? 2.0 * M * N * kdim * reps * sms / (ms * 1e-3) / 1e12 : 0.0;
    *cycles_per_mma = rc == PBR_OK ? static_cast<double>(cyc) / reps : 0.0;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}
