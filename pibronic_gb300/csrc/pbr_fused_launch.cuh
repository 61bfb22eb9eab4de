// pbr_fused_launch.cuh -- host launcher for the fused kernel, included once per surface count.
#pragma once

#include <algorithm>

#include "pbr_fused.cuh"

namespace pbr {

template <int A, int K, int QM, typename T, bool kTcq>
static int launch_fused_kern(const FusedArgs& args, cudaStream_t stream) {
    const SmemPlan plan(A, K, QM, static_cast<int>(sizeof(T)), args.m.N, args.m.P, args.S,
                        args.qstride, kTcq ? 1 : 0);
    auto kern = pimc_fused_kernel<A, K, QM, T, kTcq>;
    static int configured = 0;    // dynamic shared memory opt-in already granted to this kernel
    if (plan.total_bytes > 48 * 1024 && plan.total_bytes > configured) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 plan.total_bytes) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = plan.total_bytes;
    }
    int dev = 0, sms = 0, occ = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreads,
                                                                     plan.total_bytes));
    if (occ < 1) return PBR_ERR_UNSUPPORTED;
    const int64_t need = (args.X + args.S - 1) / args.S;
    const int grid = static_cast<int>(std::min<int64_t>(need, static_cast<int64_t>(occ) * sms));
    if (grid <= 0) return PBR_OK;
    kern<<<grid, kThreads, plan.total_bytes, stream>>>(args);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

template <int A, int K, int QM, typename T>
static int launch_fused_one(const FusedArgs& args, cudaStream_t stream) {
    if constexpr (sizeof(T) == 4 && A >= 3)
        if (args.tcq) return launch_fused_kern<A, K, QM, T, true>(args, stream);
    return launch_fused_kern<A, K, QM, T, false>(args, stream);
}

template <int A>
int launch_fused(int K, int qmode, int precision, const FusedArgs& args, cudaStream_t stream) {
    if (precision == 32) {
        if (K == 0) {
            if (qmode == kSample) return launch_fused_one<A, 0, kSample, float>(args, stream);
            if (qmode == kQ64) return launch_fused_one<A, 0, kQ64, float>(args, stream);
            return launch_fused_one<A, 0, kQ32, float>(args, stream);
        }
        if (qmode == kSample) return launch_fused_one<A, 4, kSample, float>(args, stream);
        if (qmode == kQ64) return launch_fused_one<A, 4, kQ64, float>(args, stream);
        return launch_fused_one<A, 4, kQ32, float>(args, stream);
    }
    if (qmode == kQ32) return PBR_ERR_UNSUPPORTED;
    if (K == 0) {
        if (qmode == kSample) return launch_fused_one<A, 0, kSample, double>(args, stream);
        return launch_fused_one<A, 0, kQ64, double>(args, stream);
    }
    if (qmode == kSample) return launch_fused_one<A, 4, kSample, double>(args, stream);
    return launch_fused_one<A, 4, kQ64, double>(args, stream);
}

}  // namespace pbr
