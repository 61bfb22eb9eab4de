// pbr_common.cuh -- device helpers shared by the PIMC kernels (sm_103a).
//
//  * Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
//    as easy as 1, 2, 3", SC'11): round function with the published multipliers and Weyl key
//    increments, written from the paper.
//  * Box-Muller normals.
//  * Cyclic Jacobi eigensolver for a small symmetric matrix held in registers (Golub & Van Loan,
//    "Matrix Computations", symmetric Schur rotation), templated on the scalar type and size.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/pibronic_gb300.h"

namespace pbr {

// ----------------------------------------------------------------------------------------------
// Philox4x32-10
// ----------------------------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

__device__ __forceinline__ void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = static_cast<uint64_t>(a) * static_cast<uint64_t>(b);
    hi = static_cast<uint32_t>(p >> 32);
    lo = static_cast<uint32_t>(p);
}

__device__ __forceinline__ u32x4 philox4x32_10(u32x4 ctr, uint32_t k0, uint32_t k1) {
    constexpr uint32_t kM0 = 0xD2511F53u, kM1 = 0xCD9E8D57u;   // round multipliers
    constexpr uint32_t kW0 = 0x9E3779B9u, kW1 = 0xBB67AE85u;   // key schedule (Weyl) increments
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(kM0, ctr.x, hi0, lo0);
        mulhilo(kM1, ctr.z, hi1, lo1);
        ctr = u32x4{hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0};
        k0 += kW0;
        k1 += kW1;
    }
    return ctr;
}

// uniform in the open interval (0, 1)
__device__ __forceinline__ float u01(uint32_t v) {
    return (static_cast<float>(v >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// two standard normals from two uniforms (Box-Muller), with the hardware-approximate log and
// sine / cosine: u01 keeps the log's argument in (0, 1] and the angle in (0, 2 pi), where both are
// accurate to about 1e-6 -- far below what a Gaussian draw needs, and the draws stay a function of
// the counter alone (every kernel form calls this function)
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
    const float r = sqrtf(-2.0f * __logf(u01(a)));
    float s, c;
    __sincosf(6.283185307179586f * u01(b), &s, &c);
    z0 = r * c;
    z1 = r * s;
}

// ----------------------------------------------------------------------------------------------
// small helpers
// ----------------------------------------------------------------------------------------------

// d * 2^n, exact (as ldexp) -- one FP64 multiply by a power of two built from its exponent bits
// when n is a normal exponent, ldexp otherwise
__device__ __forceinline__ double scale_pow2(double d, int n) {
    if (n >= -1022 && n <= 1023) return d * __longlong_as_double(static_cast<long long>(n + 1023) << 52);
    return ldexp(d, n);
}

// e^x for the per-sample FP64 outputs of the FP32 kernels, whose arguments are sums of FP32 terms
// (absolute error ~1e-6 and above): e^x = 2^n 2^f, n = floor(x log2 e) applied exactly and
// 2^f (0 <= f < 1) from exp2f (relative error ~2e-7); extreme or non-finite x takes exp.  A few
// FP64 operations instead of a full FP64 exponential, on a part whose FP64 rate is a small
// fraction of its FP32 rate.
__device__ __forceinline__ double exp_out_fp32(double x) {
    const double t = x * 1.4426950408889634;
    if (!(fabs(t) < 1000.0)) return exp(x);
    const double n = floor(t);
    return scale_pow2(static_cast<double>(exp2f(static_cast<float>(t - n))), static_cast<int>(n));
}
// the output exponential of a kernel computing in T: FP64 exp for the FP64 builds
template <typename T>
__device__ __forceinline__ double exp_out(double x) {
    if constexpr (sizeof(T) == 8) return exp(x);
    else return exp_out_fp32(x);
}
__host__ __device__ constexpr int npair(int n) { return n * (n + 1) / 2; }
__host__ __device__ constexpr int pair_index(int b, int c) { return b * (b + 1) / 2 + c; }  // b >= c

template <typename T> __device__ __forceinline__ T dev_exp2(T x);
template <> __device__ __forceinline__ float dev_exp2<float>(float x) { return exp2f(x); }
template <> __device__ __forceinline__ double dev_exp2<double>(double x) { return exp2(x); }

template <typename T> __device__ __forceinline__ T dev_exp(T x);
template <> __device__ __forceinline__ float dev_exp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double dev_exp<double>(double x) { return exp(x); }

template <typename T> __device__ __forceinline__ T dev_sqrt(T x);
template <> __device__ __forceinline__ float dev_sqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double dev_sqrt<double>(double x) { return sqrt(x); }

template <typename T> __device__ __forceinline__ T dev_rsqrt(T x);
template <> __device__ __forceinline__ float dev_rsqrt<float>(float x) { return rsqrtf(x); }
template <> __device__ __forceinline__ double dev_rsqrt<double>(double x) { return rsqrt(x); }

template <typename T> struct eps_of;
template <> struct eps_of<float>  { static constexpr float  value = 1.1920929e-07f; };
template <> struct eps_of<double> { static constexpr double value = 2.220446049250313e-16; };

// ----------------------------------------------------------------------------------------------
// Cyclic Jacobi on a symmetric A x A matrix a[][] (full storage, registers).  On return the
// diagonal of a holds the eigenvalues and the columns of u the eigenvectors (a = u diag u^T).
// Sweeps stop when the off-diagonal mass is below (eps * ||diag||)^2 or after max_sweeps.
// ----------------------------------------------------------------------------------------------
template <typename T, int A>
__device__ __forceinline__ void jacobi_eigh(T (&a)[A][A], T (&u)[A][A], int max_sweeps) {
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c < A; ++c) u[r][c] = (r == c) ? T(1) : T(0);
    if (A == 1) return;
    const T tol = eps_of<T>::value * eps_of<T>::value;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        T off = T(0), dia = T(0);
#pragma unroll
        for (int p = 0; p < A; ++p) {
            dia += a[p][p] * a[p][p];
#pragma unroll
            for (int q = p + 1; q < A; ++q) off += a[p][q] * a[p][q];
        }
        if (off <= tol * dia || off == T(0)) break;
#pragma unroll
        for (int p = 0; p < A - 1; ++p) {
#pragma unroll
            for (int q = p + 1; q < A; ++q) {
                const T apq = a[p][q];
                if (apq == T(0)) continue;
                const T zeta = (a[q][q] - a[p][p]) / (T(2) * apq);
                const T az = fabs(zeta);
                T t;
                if (az > T(1) / eps_of<T>::value) {
                    t = T(0.5) / zeta;                       // tiny rotation, avoids zeta^2 overflow
                } else {
                    t = T(1) / (az + dev_sqrt<T>(T(1) + zeta * zeta));
                    if (zeta < T(0)) t = -t;
                }
                const T c = dev_rsqrt<T>(T(1) + t * t);
                const T s = t * c;
                a[p][p] -= t * apq;
                a[q][q] += t * apq;
                a[p][q] = T(0);
                a[q][p] = T(0);
#pragma unroll
                for (int r = 0; r < A; ++r) {
                    if (r == p || r == q) continue;
                    const T arp = a[r][p], arq = a[r][q];
                    const T np = c * arp - s * arq;
                    const T nq = s * arp + c * arq;
                    a[r][p] = np; a[p][r] = np;
                    a[r][q] = nq; a[q][r] = nq;
                }
#pragma unroll
                for (int r = 0; r < A; ++r) {
                    const T urp = u[r][p], urq = u[r][q];
                    u[r][p] = c * urp - s * urq;
                    u[r][q] = s * urp + c * urq;
                }
            }
        }
    }
}

// ----------------------------------------------------------------------------------------------
// status helpers
// ----------------------------------------------------------------------------------------------
__device__ __forceinline__ void flag_status(int32_t* status, int32_t code) {
    if (status) atomicMax(status, code);
}

// FP16 pair (x0, x1), x0 in the low half
__device__ __forceinline__ uint32_t pack_f16x2(float x0, float x1) {
    uint32_t r;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(x1), "f"(x0));
    return r;
}

// hi = FP16(x) and lo = FP16(x - hi) for two values, packed as FP16 pairs
__device__ __forceinline__ void split_f16x2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    hi = pack_f16x2(x0, x1);
    const __half2 h = *reinterpret_cast<const __half2*>(&hi);
    const float2 hf = __half22float2(h);
    lo = pack_f16x2(x0 - hf.x, x1 - hf.y);
}

}  // namespace pbr

#define PBR_CUDA_CHECK_RET(expr)                                                                \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) return PBR_ERR_CUDA;                                             \
    } while (0)
