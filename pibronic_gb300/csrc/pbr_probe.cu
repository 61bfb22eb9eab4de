// pbr_probe.cu -- FP32 FMA throughput probe (the CUDA-core roofline denominator the fused kernel
// is measured against; it has no counterpart in the reference).
#include "pbr_common.cuh"

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float* out, int iters, float seed) {
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = seed + 0.001f * static_cast<float>(threadIdx.x + i);
    const float b = 0.999999f, c = 1e-7f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int r = 0; r < 16; ++r)
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], b, c);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += a[i];
    if (s == 12345.678f) out[blockIdx.x] = s;   // keeps the chains live
}

}  // namespace

extern "C" int pbr_fma_probe(float* out, int32_t blocks, int32_t iters, double* flops, void* stream) {
    if (!out || blocks < 1 || iters < 1) return PBR_ERR_ARG;
    fma_probe_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, iters, 1.0f);
    if (flops) *flops = 2.0 * 8.0 * 16.0 * static_cast<double>(iters) * 256.0 * blocks;
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}
