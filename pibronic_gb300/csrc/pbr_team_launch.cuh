// pbr_team_launch.cuh -- host launcher for the row-team kernel, included once per surface count.
#pragma once

#include <algorithm>

#include "pbr_team.cuh"

namespace pbr {

// the two-block build applies at 5 and 6 surfaces in FP32 when two tiles fit an SM
template <int A, typename T>
constexpr bool team_two_block_build() { return (A == 5 || A == 6) && sizeof(T) == 4; }

template <int A, int K, int QM, typename T, int MB, bool kTcq = false>
static int launch_team_kern(const TeamArgs& args, int smem_bytes, cudaStream_t stream) {
    auto kern = pimc_team_kernel<A, K, QM, T, MB, kTcq>;
    static int configured = 0;
    if (smem_bytes > 48 * 1024 && smem_bytes > configured) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = smem_bytes;
    }
    int dev = 0, sms = 0, occ = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTeamThreads, smem_bytes));
    if (occ < 1) return PBR_ERR_UNSUPPORTED;
    const int64_t need = (args.X + args.S - 1) / args.S;
    const int grid = static_cast<int>(std::min<int64_t>(need, static_cast<int64_t>(occ) * sms));
    if (grid <= 0) return PBR_OK;
    kern<<<grid, kTeamThreads, smem_bytes, stream>>>(args);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

template <int A, int K, int QM, typename T>
static int launch_team_one(const TeamArgs& args, cudaStream_t stream) {
    const TeamPlan plan(A, K, QM, static_cast<int>(sizeof(T)), args.m.N, args.m.P, args.S, args.G,
                        args.qstride, args.rl, args.tcq);
    if constexpr (sizeof(T) == 4 && QM != kQ32V && A >= 3 && team_min_blocks<A>() == 1)
        if (args.tcq) return launch_team_kern<A, K, QM, T, 1, true>(args, plan.total_bytes, stream);
    if constexpr (team_two_block_build<A, T>())
        if (plan.total_bytes <= kTeamTwoBlockSmem) return launch_team_kern<A, K, QM, T, 2>(args, plan.total_bytes, stream);
    return launch_team_kern<A, K, QM, T, team_min_blocks<A>()>(args, plan.total_bytes, stream);
}

template <int A>
int launch_team(int K, int qmode, int precision, const TeamArgs& args, cudaStream_t stream) {
    if (precision == 32) {
        if (K == 0) {
            if (qmode == kSample) return launch_team_one<A, 0, kSample, float>(args, stream);
            if (qmode == kQ64) return launch_team_one<A, 0, kQ64, float>(args, stream);
            if (qmode == kQ32V) return launch_team_one<A, 0, kQ32V, float>(args, stream);
            return launch_team_one<A, 0, kQ32, float>(args, stream);
        }
        if (qmode == kSample) return launch_team_one<A, 4, kSample, float>(args, stream);
        if (qmode == kQ64) return launch_team_one<A, 4, kQ64, float>(args, stream);
        if (qmode == kQ32V) return launch_team_one<A, 4, kQ32V, float>(args, stream);
        return launch_team_one<A, 4, kQ32, float>(args, stream);
    }
    if (qmode == kQ32 || qmode == kQ32V) return PBR_ERR_UNSUPPORTED;
    if (K == 0) {
        if (qmode == kSample) return launch_team_one<A, 0, kSample, double>(args, stream);
        return launch_team_one<A, 0, kQ64, double>(args, stream);
    }
    if (qmode == kSample) return launch_team_one<A, 4, kSample, double>(args, stream);
    return launch_team_one<A, 4, kQ64, double>(args, stream);
}

template <int A, int K, int MB, bool kTcq = false>
static int launch_team_batch_kern(const TeamBatchItem* items, int n_items, int64_t total_tiles, int smem_bytes,
                                  int grid_cap, cudaStream_t stream) {
    auto kern = pimc_team_batch_kernel<A, K, MB, kTcq>;
    if (smem_bytes > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes) != cudaSuccess)
        return PBR_ERR_UNSUPPORTED;
    int dev = 0, sms = 0, occ = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTeamThreads, smem_bytes));
    if (occ < 1) return PBR_ERR_UNSUPPORTED;
    int64_t grid = std::min<int64_t>(total_tiles, static_cast<int64_t>(occ) * sms);
    if (grid_cap > 0) grid = std::min<int64_t>(grid, grid_cap);
    if (grid <= 0) return PBR_OK;
    kern<<<static_cast<int>(grid), kTeamThreads, smem_bytes, stream>>>(items, n_items, total_tiles);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

template <int A, int K>
static int launch_team_batch_one(const TeamBatchItem* items, int n_items, int64_t total_tiles, int smem_bytes,
                                 int grid_cap, int tcq, cudaStream_t stream) {
    // a group of models on the tensor-core quadratic (one block per SM, 3+ surfaces)
    if constexpr (A >= 3 && team_min_blocks<A>() == 1)
        if (tcq) return launch_team_batch_kern<A, K, 1, true>(items, n_items, total_tiles, smem_bytes, grid_cap, stream);
    if constexpr (team_two_block_build<A, float>())
        if (smem_bytes <= kTeamTwoBlockSmem)
            return launch_team_batch_kern<A, K, 2>(items, n_items, total_tiles, smem_bytes, grid_cap, stream);
    return launch_team_batch_kern<A, K, team_min_blocks<A>()>(items, n_items, total_tiles, smem_bytes, grid_cap,
                                                              stream);
}

template <int A>
int launch_team_batch(int K, const TeamBatchItem* items, int n_items, int64_t total_tiles, int smem_bytes,
                      int grid_cap, int tcq, cudaStream_t stream) {
    if (K == 0) return launch_team_batch_one<A, 0>(items, n_items, total_tiles, smem_bytes, grid_cap, tcq, stream);
    return launch_team_batch_one<A, 4>(items, n_items, total_tiles, smem_bytes, grid_cap, tcq, stream);
}

}  // namespace pbr
