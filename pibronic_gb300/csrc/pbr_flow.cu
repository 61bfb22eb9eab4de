// pbr_flow.cu -- kernels of the learned importance proposal (affine-coupling flow over whitened
// ring normal modes).  No counterpart in the reference: Pibronic's only learned-proposal seam is
// the training-data path (pimc.py:1216-1338), which these kernels consume.
//
//   pbr_flow_prepare        q -> selected whitened normal-mode coordinates y, rest of rho's
//                           quadratic form U
//   pbr_flow_layer_forward  one coupling layer, warp per sample, weights in shared memory,
//                           either direction, optionally saving the activations for training
//   pbr_flow_layer_backward per-sample back-propagation through one layer (inverse direction)
//   pbr_gemm_tn_acc         C (+)= A^T B over the batch (weight gradients), split over the batch
//                           and reduced in a fixed order
//   pbr_colsum              column sums (bias gradients)
//   pbr_flow_base           mixture log-density of the base, responsibilities, dL/dy0
//   pbr_flow_apply          x = q + sum_s B_s sigma_s (y' - y)
//   pbr_flow_weights        proposal density of x in the scale of x's PIMC outputs
//   pbr_adam                Adam update
#include <algorithm>
#include <cmath>

#include "pbr_common.cuh"

namespace {

constexpr int kFlowWarps = 4;
constexpr float kKappa = 2.0f;

__host__ __device__ inline int align_up_(int x, int a) { return (x + a - 1) / a * a; }

// The launch helpers below cache what they ask the runtime (SM count, per-kernel residency), so a
// repeated launch -- in particular one recorded into a CUDA graph -- issues nothing but the launch.
// The caches assume one device per process (as the library does) and calls from one host thread.
inline int sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        sms = n > 0 ? n : 1;
    }
    return sms;
}

// blocks of kern resident per SM with `threads` threads and `bytes` of dynamic shared memory
// (the opt-in limit raised to the whole 227 KB once per kernel); 0 when it cannot run
template <typename K>
int resident_blocks(K kern, int threads, int bytes) {
    struct Entry { const void* f; int threads, bytes, occ; };
    static Entry cache[64];
    static int n = 0;
    const void* f = reinterpret_cast<const void*>(kern);
    bool opted = false;
    for (int i = 0; i < n; ++i) {
        if (cache[i].f != f) continue;
        opted = true;
        if (cache[i].threads == threads && cache[i].bytes == bytes) return cache[i].occ;
    }
    if (!opted && cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
        return 0;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, bytes) != cudaSuccess) return 0;
    if (n < 64) cache[n++] = Entry{f, threads, bytes, occ};
    return occ;
}

// ---------------------------------------------------------------------------------------------
// prepare: y[x][j*nsel + s] = (sum_p B_ps (q_jp - c_j)) * inv_sigma[j*nsel + s],
//          U[x] = sum_j (q_j - c_j)^T Lambda_j (q_j - c_j) - sum |y|^2
// Lambda_j = 2 coth I - csch C evaluated as sum_p csch (dx)^2 + 2 tanh(tau w/2) x_p^2.
// One thread per (sample, mode), reading the mode's P beads in order (16-byte loads when P % 4
// == 0): the ring energy and the nsel projections of the mode in FP32, no shuffles; a block holds
// whole samples (floor(blockDim / N) of them), whose modes' terms are summed in FP64 through
// shared memory.  (The warp-per-sample form with a shuffle reduction per mode took 4-5x longer.)
// ---------------------------------------------------------------------------------------------
__global__ void flow_prepare_kernel(const float* __restrict__ q, int64_t X, int N, int P, int nsel,
                                    const double* __restrict__ center, const double* __restrict__ inv_sigma,
                                    const double* __restrict__ rho_csch, const double* __restrict__ rho_tanh2,
                                    float* __restrict__ y, double* __restrict__ U) {
    extern __shared__ double part[];            // [blockDim] per-thread FP64 terms, then (FP32):
    float* basis = reinterpret_cast<float*>(part + blockDim.x);   // [nsel][P] ring basis columns
    float* s_isig = basis + nsel * P;           // inv_sigma [N][nsel]
    float* s_mode = s_isig + N * nsel;          // [N][4]: center, csch, 2 tanh(tau w / 2), 0
    const double inv_sqrt_p = 1.0 / sqrt(static_cast<double>(P));
    const double amp = sqrt(2.0 / P);
    for (int i = threadIdx.x; i < nsel * P; i += blockDim.x) {
        const int s = i / P, p = i - s * P;
        double bv = inv_sqrt_p;
        if (s > 0) {
            double sn, cs;
            sincospi(2.0 * ((s + 1) / 2) * p / P, &sn, &cs);
            bv = amp * ((s & 1) ? cs : sn);
        }
        basis[i] = static_cast<float>(bv);
    }
    for (int i = threadIdx.x; i < N * nsel; i += blockDim.x) s_isig[i] = static_cast<float>(inv_sigma[i]);
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        s_mode[4 * j] = static_cast<float>(center[j]);
        s_mode[4 * j + 1] = static_cast<float>(rho_csch[j]);
        s_mode[4 * j + 2] = static_cast<float>(2.0 * rho_tanh2[j]);
        s_mode[4 * j + 3] = 0.f;
    }
    __syncthreads();
    const int spb = static_cast<int>(blockDim.x) / N;            // whole samples per block
    const int t = threadIdx.x, sl = t / N, j = t - sl * N;
    const bool vec = (P & 3) == 0 && (reinterpret_cast<uintptr_t>(q) & 15) == 0;
    for (int64_t x0 = static_cast<int64_t>(blockIdx.x) * spb; x0 < X; x0 += static_cast<int64_t>(gridDim.x) * spb) {
        const int64_t x = x0 + sl;
        double term = 0.0;
        if (sl < spb && x < X) {
            const float* qj = q + (x * N + j) * static_cast<int64_t>(P);
            const float c = s_mode[4 * j], ch = s_mode[4 * j + 1], th2 = s_mode[4 * j + 2];
            float quad = 0.f, proj[8];
#pragma unroll
            for (int s = 0; s < 8; ++s) proj[s] = 0.f;
            const float xfirst = qj[0] - c;
            float xprev = xfirst;
            auto bead = [&](int p, float xp) {
                const float d = xprev - xp;          // x_{p-1} - x_p (the pair (p-1, p) of the ring)
                quad = fmaf(th2 * xp, xp, quad);
                if (p > 0) quad = fmaf(ch * d, d, quad);
#pragma unroll
                for (int s = 0; s < 8; ++s)
                    if (s < nsel) proj[s] = fmaf(basis[s * P + p], xp, proj[s]);
                xprev = xp;
            };
            if (vec) {
                const float4* q4 = reinterpret_cast<const float4*>(qj);
                for (int p4 = 0; p4 < P / 4; ++p4) {
                    const float4 v = q4[p4];
                    bead(4 * p4, v.x - c);
                    bead(4 * p4 + 1, v.y - c);
                    bead(4 * p4 + 2, v.z - c);
                    bead(4 * p4 + 3, v.w - c);
                }
            } else {
                for (int p = 0; p < P; ++p) bead(p, qj[p] - c);
            }
            {
                const float d = xprev - xfirst;      // the ring's closing pair (P-1, 0)
                quad = fmaf(ch * d, d, quad);
            }
            float ysq = 0.f;
            float* yo = y + x * static_cast<int64_t>(N * nsel) + j * nsel;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                if (s >= nsel) break;
                const float v = proj[s] * s_isig[j * nsel + s];
                ysq = fmaf(v, v, ysq);
                yo[s] = v;
            }
            term = static_cast<double>(quad) - static_cast<double>(ysq);
        }
        part[t] = term;
        __syncthreads();
        if (t < spb && x0 + t < X) {
            double sum = 0.0;
            for (int jj = 0; jj < N; ++jj) sum += part[t * N + jj];
            U[x0 + t] = sum;
        }
        __syncthreads();
    }
}

// x = q + sum_{s < nsel} B_ps sigma_js (y'_js - y_js)
// A warp takes kApplyRows (sample, mode) rows at a time: their nsel displacements in one load per
// lane, then lanes over the beads of all the rows together (coalesced, kApplyRows loads in flight
// per lane).  (A warp per row, waiting on the row's displacements before its beads, reached 2.9
// TB/s.)
constexpr int kApplyRows = 4;

__global__ void __launch_bounds__(256) flow_apply_kernel(const float* __restrict__ q, const float* __restrict__ y,
                                                         const float* __restrict__ yn, int64_t X, int N, int P,
                                                         int nsel, const double* __restrict__ sigma,
                                                         float* __restrict__ xo) {
    extern __shared__ float basis[];            // [nsel][P], then sigma [N][nsel] in FP32
    float* s_sig = basis + nsel * P;
    const double inv_sqrt_p = 1.0 / sqrt(static_cast<double>(P));
    const double amp = sqrt(2.0 / P);
    for (int i = threadIdx.x; i < nsel * P; i += blockDim.x) {
        const int s = i / P, p = i - s * P;
        double bv = inv_sqrt_p;
        if (s > 0) {
            double sn, cs;
            sincospi(2.0 * ((s + 1) / 2) * p / P, &sn, &cs);
            bv = amp * ((s & 1) ? cs : sn);
        }
        basis[i] = static_cast<float>(bv);
    }
    for (int i = threadIdx.x; i < N * nsel; i += blockDim.x) s_sig[i] = static_cast<float>(sigma[i]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t rows = X * N;
    const int64_t w0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t r0 = w0 * kApplyRows; r0 < rows; r0 += nw * kApplyRows) {
        // lane l < kApplyRows nsel: the displacement of row r0 + l / nsel, slot l % nsel
        float dv = 0.f;
        if (lane < kApplyRows * nsel) {
            const int64_t row = r0 + lane / nsel;
            const int s = lane % nsel;
            if (row < rows) {
                const int j = static_cast<int>(row % N);
                dv = s_sig[j * nsel + s] * (yn[row * nsel + s] - y[row * nsel + s]);
            }
        }
        float dy[kApplyRows][8];
#pragma unroll
        for (int k = 0; k < kApplyRows; ++k)
#pragma unroll
            for (int s = 0; s < 8; ++s) dy[k][s] = __shfl_sync(0xffffffffu, dv, (k * nsel + s) & 31);
        const int nr = static_cast<int>(min(static_cast<int64_t>(kApplyRows), rows - r0));
        for (int p = lane; p < P; p += 32) {
            float b[8];
#pragma unroll
            for (int s = 0; s < 8; ++s) b[s] = s < nsel ? basis[s * P + p] : 0.f;
            float v[kApplyRows];
#pragma unroll
            for (int k = 0; k < kApplyRows; ++k) v[k] = k < nr ? q[(r0 + k) * P + p] : 0.f;
#pragma unroll
            for (int k = 0; k < kApplyRows; ++k) {
                float acc = v[k];
#pragma unroll
                for (int s = 0; s < 8; ++s)
                    if (s < nsel) acc = fmaf(b[s], dy[k][s], acc);
                if (k < nr) xo[(r0 + k) * P + p] = acc;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// coupling layer, warp per sample.  Shared memory: W1 [I][H], W2 [H][H], W3 [H][2J], biases,
// then per-warp buffers ya[I], h1[H], h2[H].
// ---------------------------------------------------------------------------------------------
struct LayerDev {
    int D, I, J, H;
    const int32_t* idx_a;
    const int32_t* idx_b;
    const float* W1; const float* b1; const float* W2; const float* b2; const float* W3; const float* b3;
};

struct SaveDev {
    float* ya; float* h1; float* h2; float* s; float* yb;   // each nullable (all or none)
};

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// UPH consecutive floats from shared memory (UPH in {1, 2, 4, 8}), vector loads
template <int UPH>
__device__ __forceinline__ void ldu(const float* __restrict__ p, float (&v)[UPH]) {
    if constexpr (UPH % 4 == 0) {
#pragma unroll
        for (int u = 0; u < UPH; u += 4) {
            const float4 t = *reinterpret_cast<const float4*>(p + u);
            v[u] = t.x; v[u + 1] = t.y; v[u + 2] = t.z; v[u + 3] = t.w;
        }
    } else if constexpr (UPH == 2) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
        v[0] = p[0];
    }
}

// Layer in either direction.  Lane l owns hidden units [l*UPH, (l+1)*UPH); the output head
// pairs (s_j, t_j) belong to lane j mod 32; k-sums are split in four interleaved partials.
template <int UPH>
__global__ void flow_layer_fwd_kernel(const LayerDev L, int dir, int64_t X, float* __restrict__ y,
                                      double* __restrict__ logdet, const SaveDev sv) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D, O = 2 * J;
    float* w1 = fsm;                       // [I][H]
    float* w2 = w1 + I * H;                // [H][H]
    float* w3 = w2 + H * H;                // [H][O]
    float* bb1 = w3 + H * O;
    float* bb2 = bb1 + H;
    float* bb3 = bb2 + H;
    float* wbuf = bb3 + align_up_(O, 4);
    for (int i = threadIdx.x; i < I * H; i += blockDim.x) w1[i] = L.W1[i];
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) w2[i] = L.W2[i];
    for (int i = threadIdx.x; i < H * O; i += blockDim.x) w3[i] = L.W3[i];
    for (int i = threadIdx.x; i < H; i += blockDim.x) { bb1[i] = L.b1[i]; bb2[i] = L.b2[i]; }
    for (int i = threadIdx.x; i < O; i += blockDim.x) bb3[i] = L.b3[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int WB = align_up_(I, 4) + 2 * H;
    float* ya = wbuf + warp * WB;
    float* h1 = ya + align_up_(I, 4);
    float* h2 = h1 + H;
    const int h0 = lane * UPH;
    const int64_t nw = static_cast<int64_t>(gridDim.x) * kFlowWarps;
    for (int64_t x = static_cast<int64_t>(blockIdx.x) * kFlowWarps + warp; x < X; x += nw) {
        float* yx = y + x * D;
        for (int i = lane; i < I; i += 32) ya[i] = yx[L.idx_a[i]];
        __syncwarp();
        {
            float acc[UPH], w[UPH];
            ldu<UPH>(bb1 + h0, acc);
            for (int i = 0; i < I; ++i) {
                const float a = ya[i];
                ldu<UPH>(w1 + i * H + h0, w);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[u] = fmaf(a, w[u], acc[u]);
            }
#pragma unroll
            for (int u = 0; u < UPH; ++u) h1[h0 + u] = tanhf(acc[u]);
        }
        __syncwarp();
        {
            float acc[2][UPH], w[UPH];
            ldu<UPH>(bb2 + h0, acc[0]);
#pragma unroll
            for (int u = 0; u < UPH; ++u) acc[1][u] = 0.f;
            for (int k = 0; k < H; k += 2) {
                const float a0 = h1[k], a1 = h1[k + 1];
                ldu<UPH>(w2 + k * H + h0, w);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[0][u] = fmaf(a0, w[u], acc[0][u]);
                ldu<UPH>(w2 + (k + 1) * H + h0, w);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[1][u] = fmaf(a1, w[u], acc[1][u]);
            }
#pragma unroll
            for (int u = 0; u < UPH; ++u) h2[h0 + u] = tanhf(acc[0][u] + acc[1][u]);
        }
        __syncwarp();
        float ssum = 0.0f;
        for (int j = lane; j < J; j += 32) {
            float os[4] = {bb3[j], 0.f, 0.f, 0.f}, ot[4] = {bb3[J + j], 0.f, 0.f, 0.f};
            for (int k = 0; k < H; k += 4) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float hk = h2[k + u];
                    os[u] = fmaf(hk, w3[(k + u) * O + j], os[u]);
                    ot[u] = fmaf(hk, w3[(k + u) * O + J + j], ot[u]);
                }
            }
            const float so = (os[0] + os[1]) + (os[2] + os[3]);
            const float to = (ot[0] + ot[1]) + (ot[2] + ot[3]);
            const float sv_s = kKappa * tanhf(so / kKappa);
            const int bi = L.idx_b[j];
            const float yb = yx[bi];
            const float out = (dir > 0) ? fmaf(yb, __expf(sv_s), to) : (yb - to) * __expf(-sv_s);
            yx[bi] = out;
            ssum += sv_s;
            if (sv.s) { sv.s[x * J + j] = sv_s; sv.yb[x * J + j] = out; }
        }
        ssum = warp_sum(ssum);
        if (lane == 0) logdet[x] += (dir > 0) ? static_cast<double>(ssum) : -static_cast<double>(ssum);
        if (sv.ya) {
            for (int i = lane; i < I; i += 32) sv.ya[x * I + i] = ya[i];
            for (int h = lane; h < H; h += 32) { sv.h1[x * H + h] = h1[h]; sv.h2[x * H + h] = h2[h]; }
        }
        __syncwarp();
    }
}

// Back-propagation through one layer of the inverse direction.  gy holds dL/dy of the layer's
// output on entry and dL/dy' of its input on exit; g_o [X][2J], g_z2 / g_z1 [X][H] are written
// for the weight-gradient GEMMs.  rt[x] is the sample's normalised weight (the log-det term).
template <int UPH>
__global__ void flow_layer_bwd_kernel(const LayerDev L, int64_t X, float* __restrict__ gy,
                                      const float* __restrict__ rt, const SaveDev sv,
                                      float* __restrict__ g_o, float* __restrict__ g_z2,
                                      float* __restrict__ g_z1) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D, O = 2 * J;
    const int IP = align_up_(I, 32);
    float* w1t = fsm;                 // [H][IP]  W1 transposed
    float* w2t = w1t + H * IP;        // [H][H]   W2 transposed
    float* w3t = w2t + H * H;         // [O][H]   W3 transposed
    float* wbuf = w3t + O * H;
    for (int i = threadIdx.x; i < H * IP; i += blockDim.x) {
        const int k = i / IP, r = i - k * IP;
        w1t[i] = (r < I) ? L.W1[r * H + k] : 0.f;
    }
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) {
        const int r = i / H, c = i - r * H;
        w2t[c * H + r] = L.W2[i];
    }
    for (int i = threadIdx.x; i < H * O; i += blockDim.x) {
        const int r = i / O, c = i - r * O;
        w3t[c * H + r] = L.W3[i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int WB = align_up_(O, 4) + 2 * H;
    float* go = wbuf + warp * WB;
    float* gz2 = go + align_up_(O, 4);
    float* gz1 = gz2 + H;
    const int h0 = lane * UPH;
    const int64_t nw = static_cast<int64_t>(gridDim.x) * kFlowWarps;
    for (int64_t x = static_cast<int64_t>(blockIdx.x) * kFlowWarps + warp; x < X; x += nw) {
        float* gx = gy + x * D;
        const float w = rt[x];
        for (int j = lane; j < J; j += 32) {
            const int bi = L.idx_b[j];
            const float s = sv.s[x * J + j], yb = sv.yb[x * J + j];
            const float gyb = gx[bi];
            const float es = __expf(-s);
            const float gs = -gyb * yb + w;
            const float gos = gs * (1.0f - (s / kKappa) * (s / kKappa));
            const float gt = -gyb * es;
            gx[bi] = gyb * es;
            go[j] = gos;
            go[J + j] = gt;
            g_o[x * O + j] = gos;
            g_o[x * O + J + j] = gt;
        }
        __syncwarp();
        {
            float acc[2][UPH], wv[UPH], hv[UPH];
#pragma unroll
            for (int u = 0; u < UPH; ++u) { acc[0][u] = 0.f; acc[1][u] = 0.f; }
            int c = 0;
            for (; c + 1 < O; c += 2) {
                const float a0 = go[c], a1 = go[c + 1];
                ldu<UPH>(w3t + c * H + h0, wv);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[0][u] = fmaf(a0, wv[u], acc[0][u]);
                ldu<UPH>(w3t + (c + 1) * H + h0, wv);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[1][u] = fmaf(a1, wv[u], acc[1][u]);
            }
            if (c < O) {
                const float a0 = go[c];
                ldu<UPH>(w3t + c * H + h0, wv);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[0][u] = fmaf(a0, wv[u], acc[0][u]);
            }
            const float* h2x = sv.h2 + x * H + h0;
#pragma unroll
            for (int u = 0; u < UPH; ++u) hv[u] = h2x[u];
#pragma unroll
            for (int u = 0; u < UPH; ++u) {
                const float v = (acc[0][u] + acc[1][u]) * (1.0f - hv[u] * hv[u]);
                gz2[h0 + u] = v;
                g_z2[x * H + h0 + u] = v;
            }
        }
        __syncwarp();
        {
            float acc[2][UPH], wv[UPH], hv[UPH];
#pragma unroll
            for (int u = 0; u < UPH; ++u) { acc[0][u] = 0.f; acc[1][u] = 0.f; }
            for (int m = 0; m < H; m += 2) {
                const float a0 = gz2[m], a1 = gz2[m + 1];
                ldu<UPH>(w2t + m * H + h0, wv);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[0][u] = fmaf(a0, wv[u], acc[0][u]);
                ldu<UPH>(w2t + (m + 1) * H + h0, wv);
#pragma unroll
                for (int u = 0; u < UPH; ++u) acc[1][u] = fmaf(a1, wv[u], acc[1][u]);
            }
            const float* h1x = sv.h1 + x * H + h0;
#pragma unroll
            for (int u = 0; u < UPH; ++u) hv[u] = h1x[u];
#pragma unroll
            for (int u = 0; u < UPH; ++u) {
                const float v = (acc[0][u] + acc[1][u]) * (1.0f - hv[u] * hv[u]);
                gz1[h0 + u] = v;
                g_z1[x * H + h0 + u] = v;
            }
        }
        __syncwarp();
        for (int i = lane; i < I; i += 32) {
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
            for (int k = 0; k < H; k += 4) {
#pragma unroll
                for (int u = 0; u < 4; ++u) acc[u] = fmaf(gz1[k + u], w1t[(k + u) * IP + i], acc[u]);
            }
            gx[L.idx_a[i]] += (acc[0] + acc[1]) + (acc[2] + acc[3]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------------------
// Sample-tiled coupling layers (the form used whenever the padded weights fit in shared memory).
// A block takes 64 samples at a time and runs the conditioner's three dense layers as
// register-blocked shared-memory GEMMs: 16 x 16 threads, each owning 4 samples x 4*CB columns of
// a 64*CB-wide column block, so one 128-bit load of activations and CB 128-bit loads of weights
// feed 16*CB FMAs.  Weights stay resident, zero-padded: hidden width Hp = roundup(H, 64*HB)
// (HB = 1 or 2, H <= 128), head width Op = roundup(2J, 64) with the columns of s_j and t_j
// interleaved (2j, 2j+1) so a thread holds both halves of its coupling pairs.  Activation tiles
// are row-major with a row stride of 4 mod 8 floats: the two sample rows a warp reads at once fall
// in different banks.
// ---------------------------------------------------------------------------------------------
constexpr int kTileS = 64;
constexpr int kTileThreads = 256;

struct TileDims {
    int I4, Hp, Op, Ip, ldya, ldh, ldo;
    __host__ __device__ TileDims(int I, int J, int H, int HB)
        : I4(align_up_(I, 4)), Hp(align_up_(H, 64 * HB)), Op(align_up_(2 * J, 64)), Ip(align_up_(I, 64)),
          ldya(align_up_(align_up_(I, 4), 8) + 4), ldh(align_up_(H, 64 * HB) + 4), ldo(align_up_(2 * J, 64) + 4) {}
    // + the two index lists (int32) at the end
    __host__ __device__ int fwd_floats(int I, int J) const {
        return I4 * Hp + Hp * Hp + Hp * Op + 2 * Hp + Op + kTileS * (ldya + ldh) + align_up_(I + J, 4);
    }
    __host__ __device__ int bwd_floats(int I, int J) const {
        return Op * Hp + Hp * Hp + Hp * Ip + kTileS * (ldo + ldh) + align_up_(I + J, 4);
    }
};

// store(i, load(i)) for i < n over the block with eight independent loads in flight per thread
// before their stores (a plain loop keeps one global load outstanding per thread, and the
// weight preload of a launch is then bound by memory latency)
template <typename L, typename S>
__device__ __forceinline__ void block_copy(int n, L&& load, S&& store) {
    constexpr int U = 8;
    for (int b = threadIdx.x; b < n; b += U * blockDim.x) {
        float v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = b + u * blockDim.x;
            v[u] = i < n ? load(i) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = b + u * blockDim.x;
            if (i < n) store(i, v[u]);
        }
    }
}

__device__ __forceinline__ float f4c(const float4& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// acc[r][4u + v] += sum_{k < K4} in[(4 sg + r) ld_in + k] * w[k ld_w + c0 + 4 cg + 64 u + v]
template <int CB>
__device__ __forceinline__ void tile_gemm(const float* __restrict__ in, int ld_in, int K4,
                                          const float* __restrict__ w, int ld_w, int c0, int sg, int cg,
                                          float (&acc)[4][4 * CB]) {
    const float* a_row = in + 4 * sg * ld_in;
    const float* w_col = w + c0 + 4 * cg;
#pragma unroll 2
    for (int k = 0; k < K4; k += 4) {
        float4 a[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r] = *reinterpret_cast<const float4*>(a_row + r * ld_in + k);
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
            for (int u = 0; u < CB; ++u) {
                const float4 wv = *reinterpret_cast<const float4*>(w_col + (k + kk) * ld_w + 64 * u);
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const float av = f4c(a[r], kk);
                    acc[r][4 * u + 0] = fmaf(av, wv.x, acc[r][4 * u + 0]);
                    acc[r][4 * u + 1] = fmaf(av, wv.y, acc[r][4 * u + 1]);
                    acc[r][4 * u + 2] = fmaf(av, wv.z, acc[r][4 * u + 2]);
                    acc[r][4 * u + 3] = fmaf(av, wv.w, acc[r][4 * u + 3]);
                }
            }
        }
    }
}

template <int CB>
__device__ __forceinline__ void tile_init(float (&acc)[4][4 * CB], const float* __restrict__ bias, int c0, int cg) {
#pragma unroll
    for (int u = 0; u < CB; ++u) {
        const float4 b = bias ? *reinterpret_cast<const float4*>(bias + c0 + 4 * cg + 64 * u)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            acc[r][4 * u + 0] = b.x; acc[r][4 * u + 1] = b.y; acc[r][4 * u + 2] = b.z; acc[r][4 * u + 3] = b.w;
        }
    }
}

template <int HB>
__global__ void __launch_bounds__(kTileThreads) flow_tile_fwd_kernel(const LayerDev L, int dir, int64_t X,
                                                                     float* __restrict__ y,
                                                                     double* __restrict__ logdet,
                                                                     const SaveDev sv) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D;
    const TileDims td(I, J, H, HB);
    const int Hp = td.Hp, Op = td.Op, I4 = td.I4, ldya = td.ldya, ldh = td.ldh;
    float* w1 = fsm;                      // [I4][Hp]
    float* w2 = w1 + I4 * Hp;             // [Hp][Hp]
    float* w3 = w2 + Hp * Hp;             // [Hp][Op], (s_j, t_j) at columns (2j, 2j+1)
    float* bb1 = w3 + Hp * Op;
    float* bb2 = bb1 + Hp;
    float* bb3 = bb2 + Hp;                // [Op], interleaved like w3
    float* ya = bb3 + Op;                 // [64][ldya]
    float* hs = ya + kTileS * ldya;       // [64][ldh]: h1, then h2
    int* ia = reinterpret_cast<int*>(hs + kTileS * ldh);   // idx_a [I], idx_b [J]
    int* ib = ia + I;
    for (int i = threadIdx.x; i < I + J; i += blockDim.x) ia[i] = i < I ? L.idx_a[i] : L.idx_b[i - I];
    block_copy(I4 * Hp, [&](int i) { const int k = i / Hp, c = i - k * Hp;
                                     return (k < I && c < H) ? L.W1[k * H + c] : 0.f; },
               [&](int i, float v) { w1[i] = v; });
    block_copy(Hp * Hp, [&](int i) { const int k = i / Hp, c = i - k * Hp;
                                     return (k < H && c < H) ? L.W2[k * H + c] : 0.f; },
               [&](int i, float v) { w2[i] = v; });
    block_copy(Hp * Op, [&](int i) { const int k = i / Op, c = i - k * Op, j = c >> 1;
                                     return (k < H && j < J) ? L.W3[k * 2 * J + ((c & 1) ? J + j : j)] : 0.f; },
               [&](int i, float v) { w3[i] = v; });
    block_copy(2 * Hp, [&](int i) { return i < Hp ? (i < H ? L.b1[i] : 0.f) : (i - Hp < H ? L.b2[i - Hp] : 0.f); },
               [&](int i, float v) { bb1[i] = v; });                 // bb1 and bb2 are adjacent
    block_copy(Op, [&](int i) { const int j = i >> 1; return j < J ? L.b3[(i & 1) ? J + j : j] : 0.f; },
               [&](int i, float v) { bb3[i] = v; });
    const int sg = threadIdx.x >> 4, cg = threadIdx.x & 15;
    const int64_t ntiles = (X + kTileS - 1) / kTileS;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t x0 = t * kTileS;
        __syncthreads();                  // weights loaded / the previous tile's readers are done
        block_copy(kTileS * I4, [&](int i) { const int s = i / I4, c = i - s * I4; const int64_t x = x0 + s;
                                             return (c < I && x < X) ? y[x * D + ia[c]] : 0.f; },
                   [&](int i, float v) { const int s = i / I4; ya[s * ldya + (i - s * I4)] = v; });
        __syncthreads();
        if (sv.ya) {
            for (int i = threadIdx.x; i < kTileS * I; i += blockDim.x) {
                const int s = i / I, c = i - s * I;
                if (x0 + s < X) sv.ya[(x0 + s) * I + c] = ya[s * ldya + c];
            }
        }
        float acc[4][4 * HB];
        // ---- h1 = tanh(ya W1 + b1) ----
        tile_init<HB>(acc, bb1, 0, cg);
        tile_gemm<HB>(ya, ldya, I4, w1, Hp, 0, sg, cg, acc);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t x = x0 + 4 * sg + r;
#pragma unroll
            for (int u = 0; u < HB; ++u) {
                const int c = 4 * cg + 64 * u;
                const float4 h = make_float4(tanhf(acc[r][4 * u]), tanhf(acc[r][4 * u + 1]),
                                             tanhf(acc[r][4 * u + 2]), tanhf(acc[r][4 * u + 3]));
                *reinterpret_cast<float4*>(hs + (4 * sg + r) * ldh + c) = h;
                if (sv.h1 && x < X && c < H) *reinterpret_cast<float4*>(sv.h1 + x * H + c) = h;
            }
        }
        __syncthreads();
        // ---- h2 = tanh(h1 W2 + b2) ----
        tile_init<HB>(acc, bb2, 0, cg);
        tile_gemm<HB>(hs, ldh, Hp, w2, Hp, 0, sg, cg, acc);
        __syncthreads();                  // every read of h1 is done
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t x = x0 + 4 * sg + r;
#pragma unroll
            for (int u = 0; u < HB; ++u) {
                const int c = 4 * cg + 64 * u;
                const float4 h = make_float4(tanhf(acc[r][4 * u]), tanhf(acc[r][4 * u + 1]),
                                             tanhf(acc[r][4 * u + 2]), tanhf(acc[r][4 * u + 3]));
                *reinterpret_cast<float4*>(hs + (4 * sg + r) * ldh + c) = h;
                if (sv.h2 && x < X && c < H) *reinterpret_cast<float4*>(sv.h2 + x * H + c) = h;
            }
        }
        __syncthreads();
        // ---- head (s, t) = h2 W3 + b3 and the affine coupling of the b half ----
        float lsum[4] = {0.f, 0.f, 0.f, 0.f};
        for (int cb = 0; cb < Op; cb += 64) {
            float o[4][4];
            tile_init<1>(o, bb3, cb, cg);
            tile_gemm<1>(hs, ldh, Hp, w3, Op, cb, sg, cg, o);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int64_t x = x0 + 4 * sg + r;
                if (x >= X) continue;
#pragma unroll
                for (int pp = 0; pp < 2; ++pp) {
                    const int j = (cb >> 1) + 2 * cg + pp;
                    if (j >= J) continue;
                    const float sv_s = kKappa * tanhf(o[r][2 * pp] / kKappa);
                    const float to = o[r][2 * pp + 1];
                    const int bi = ib[j];
                    const float yb = y[x * D + bi];
                    const float out = (dir > 0) ? fmaf(yb, __expf(sv_s), to) : (yb - to) * __expf(-sv_s);
                    y[x * D + bi] = out;
                    lsum[r] += sv_s;
                    if (sv.s) { sv.s[x * J + j] = sv_s; sv.yb[x * J + j] = out; }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int o = 8; o >= 1; o >>= 1) lsum[r] += __shfl_xor_sync(0xffffffffu, lsum[r], o);
        if (cg == 0) {
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int64_t x = x0 + 4 * sg + r;
                if (x < X) logdet[x] += (dir > 0) ? static_cast<double>(lsum[r]) : -static_cast<double>(lsum[r]);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Training-step layers on the tensor cores (hidden width 128, I <= 64, 2J <= 64): the tile's
// GEMMs by mma.sync m16n8k16 with BF16 operands, each operand split into BF16 hi and lo parts
// (16 mantissa bits) and three MMAs per step (hi hi, hi lo, lo hi), FP32 accumulation -- about
// 1e-5 relative, well inside what the optimiser needs.  The weights sit in shared memory
// transposed, as BF16 hi and lo pairs along K (the layout of a B fragment); activations stay FP32
// in shared memory and are split when a fragment is loaded.  8 warps: warp w computes rows
// 16 (w % 4) .. + 15 and one half of the output columns.
// ---------------------------------------------------------------------------------------------
constexpr int kMmaH = 128;
struct MmaDims {
    int K1, ldw1, ldw2, Op, ldw3, ldya, ldh;
    __host__ __device__ MmaDims(int I, int J)
        : K1((I + 15) / 16 * 16), ldw1((I + 15) / 16 * 8 + 4), ldw2(kMmaH / 2 + 4), Op(64), ldw3(kMmaH / 2 + 4),
          ldya((I + 15) / 16 * 16 + 8), ldh(kMmaH + 8) {}
    // 32-bit words: W1^T, W2^T, W3^T hi and lo; biases; the ya and h tiles; row sums; index lists
    __host__ __device__ int fwd_words(int I, int J) const {
        return 2 * (kMmaH * ldw1 + kMmaH * ldw2 + Op * ldw3) + 2 * kMmaH + Op + kTileS * (ldya + ldh) +
               2 * kTileS + ((I + J + 3) / 4) * 4;
    }
};

// BF16 pair (x0 low, x1 high) rounded to nearest, and the pair of residuals
__device__ __forceinline__ void split_bf16x2(float x0, float x1, uint32_t& hi, uint32_t& lo) {
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(x1), "f"(x0));
    const float h0 = __uint_as_float(hi << 16), h1 = __uint_as_float(hi & 0xffff0000u);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(x1 - h1), "f"(x0 - h0));
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[nt] += A (64 x 16 ksteps, FP32 rows of lda) x W (W^T as BF16 pairs: wh / wl [n][ldw]) for
// this warp's 16 rows and NT n-tiles from column n0 (element (row g / g + 8, columns 2t, 2t + 1))
template <int NT>
__device__ __forceinline__ void mma_tile(const float* __restrict__ A, int lda, int ksteps,
                                         const uint32_t* __restrict__ wh, const uint32_t* __restrict__ wl,
                                         int ldw, int n0, float (&acc)[NT][4]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const float* a0 = A + (16 * (warp & 3) + g) * lda + 2 * t;
    for (int kk = 0; kk < ksteps; ++kk) {
        const float2 x0 = *reinterpret_cast<const float2*>(a0 + 16 * kk);
        const float2 x1 = *reinterpret_cast<const float2*>(a0 + 8 * lda + 16 * kk);
        const float2 x2 = *reinterpret_cast<const float2*>(a0 + 16 * kk + 8);
        const float2 x3 = *reinterpret_cast<const float2*>(a0 + 8 * lda + 16 * kk + 8);
        uint32_t ah[4], al[4];
        split_bf16x2(x0.x, x0.y, ah[0], al[0]);
        split_bf16x2(x1.x, x1.y, ah[1], al[1]);
        split_bf16x2(x2.x, x2.y, ah[2], al[2]);
        split_bf16x2(x3.x, x3.y, ah[3], al[3]);
        uint32_t bh[NT][2], bl[NT][2];
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const int o = (n0 + 8 * nt + g) * ldw + 8 * kk + t;
            bh[nt][0] = wh[o]; bh[nt][1] = wh[o + 4];
            bl[nt][0] = wl[o]; bl[nt][1] = wl[o + 4];
        }
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16_16816(acc[nt], ah, bh[nt][0], bh[nt][1]);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16_16816(acc[nt], ah, bl[nt][0], bl[nt][1]);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16_16816(acc[nt], al, bh[nt][0], bh[nt][1]);
    }
}

// B [k][n] (get(k, n); entries outside the matrix zero) as BF16 hi / lo pairs along k in rows n of
// wh / wl.  kNFast: consecutive threads take consecutive n (get reads a row-major B's rows
// contiguously), else consecutive k pairs; eight pairs per thread per round with their sixteen
// loads issued before any conversion (the staging is bound by L2 latency, not bandwidth).
template <bool kNFast, typename Get>
__device__ __forceinline__ void stage_wt(int nrows, int kpairs, int ldw, uint32_t* wh, uint32_t* wl, Get&& get) {
    constexpr int U = 8;
    const int total = nrows * kpairs;
    for (int b = threadIdx.x; b < total; b += U * blockDim.x) {
        float v0[U], v1[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = b + u * blockDim.x;
            const int n = kNFast ? i % nrows : i / kpairs, kp = kNFast ? i / nrows : i % kpairs;
            v0[u] = i < total ? get(2 * kp, n) : 0.f;
            v1[u] = i < total ? get(2 * kp + 1, n) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = b + u * blockDim.x;
            if (i >= total) continue;
            const int n = kNFast ? i % nrows : i / kpairs, kp = kNFast ? i / nrows : i % kpairs;
            uint32_t h, l;
            split_bf16x2(v0[u], v1[u], h, l);
            wh[n * ldw + kp] = h;
            wl[n * ldw + kp] = l;
        }
    }
}

// The training direction's forward pass of one layer (dir = -1 with saves) on the tensor cores;
// same outputs, saves and log-determinant updates as flow_tile_fwd_kernel.
__global__ void __launch_bounds__(kTileThreads) flow_tile_fwd_mma_kernel(const LayerDev L, int dir, int64_t X,
                                                                         float* __restrict__ y,
                                                                         double* __restrict__ logdet,
                                                                         const SaveDev sv) {
    extern __shared__ __align__(16) uint32_t msm[];
    const int I = L.I, J = L.J, D = L.D, H = kMmaH;
    const MmaDims md(I, J);
    const int K1 = md.K1, ldya = md.ldya, ldh = md.ldh;
    uint32_t* w1h = msm;                        // [H][ldw1]
    uint32_t* w1l = w1h + H * md.ldw1;
    uint32_t* w2h = w1l + H * md.ldw1;          // [H][ldw2]
    uint32_t* w2l = w2h + H * md.ldw2;
    uint32_t* w3h = w2l + H * md.ldw2;          // [Op][ldw3]: row 2j + (0: s_j, 1: t_j)
    uint32_t* w3l = w3h + md.Op * md.ldw3;
    float* bb1 = reinterpret_cast<float*>(w3l + md.Op * md.ldw3);
    float* bb2 = bb1 + H;
    float* bb3 = bb2 + H;                       // [Op], interleaved like w3
    float* ya = bb3 + md.Op;                    // [64][ldya]
    float* hs = ya + kTileS * ldya;             // [64][ldh]: h1, then h2
    float* rsum = hs + kTileS * ldh;            // [2][64]: the two column halves' sums of s per row
    int* ia = reinterpret_cast<int*>(rsum + 2 * kTileS);
    int* ib = ia + I;
    for (int i = threadIdx.x; i < I + J; i += blockDim.x) ia[i] = i < I ? L.idx_a[i] : L.idx_b[i - I];
    stage_wt<true>(H, K1 / 2, md.ldw1, w1h, w1l, [&](int k, int n) { return k < I ? L.W1[k * H + n] : 0.f; });
    stage_wt<true>(H, H / 2, md.ldw2, w2h, w2l, [&](int k, int n) { return L.W2[k * H + n]; });
    stage_wt<true>(md.Op, H / 2, md.ldw3, w3h, w3l, [&](int k, int c) {
        const int j = c >> 1;
        return j < J ? L.W3[k * 2 * J + ((c & 1) ? J + j : j)] : 0.f;
    });
    for (int i = threadIdx.x; i < 2 * H; i += blockDim.x) bb1[i] = i < H ? L.b1[i] : L.b2[i - H];
    for (int i = threadIdx.x; i < md.Op; i += blockDim.x) {
        const int j = i >> 1;
        bb3[i] = j < J ? L.b3[(i & 1) ? J + j : j] : 0.f;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int r0 = 16 * (warp & 3) + g;          // this thread's rows r0, r0 + 8
    const int half = warp >> 2;
    const int64_t ntiles = (X + kTileS - 1) / kTileS;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t x0 = tile * kTileS;
        __syncthreads();                         // weights staged / the previous tile's readers are done
        // the a half gathered: eight loads per thread issued before the stores
        for (int b = threadIdx.x; b < kTileS * K1; b += 8 * blockDim.x) {
            float v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = b + u * blockDim.x, s = i / K1, c = i - s * K1;
                const int64_t x = x0 + s;
                v[u] = (i < kTileS * K1 && c < I && x < X) ? y[x * D + ia[c]] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = b + u * blockDim.x, s = i / K1, c = i - s * K1;
                if (i >= kTileS * K1) continue;
                ya[s * ldya + c] = v[u];
                const int64_t x = x0 + s;
                if (sv.ya && c < I && x < X) sv.ya[x * I + c] = v[u];
            }
        }
        __syncthreads();
        // ---- h1 = tanh(ya W1 + b1), h2 = tanh(h1 W2 + b2): 64 columns per warp ----
        for (int layer = 0; layer < 2; ++layer) {
            const int n0 = 64 * half;
            const float* bias = layer == 0 ? bb1 : bb2;
            float acc[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const float b0 = bias[n0 + 8 * nt + 2 * t], b1 = bias[n0 + 8 * nt + 2 * t + 1];
                acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
            }
            if (layer == 0) mma_tile<8>(ya, ldya, K1 / 16, w1h, w1l, md.ldw1, n0, acc);
            else mma_tile<8>(hs, ldh, H / 16, w2h, w2l, md.ldw2, n0, acc);
            if (layer == 1) __syncthreads();      // every read of h1 is done
            float* save = layer == 0 ? sv.h1 : sv.h2;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = r0 + 8 * hh, c = n0 + 8 * nt + 2 * t;
                    const float2 h = make_float2(tanhf(acc[nt][2 * hh]), tanhf(acc[nt][2 * hh + 1]));
                    *reinterpret_cast<float2*>(hs + r * ldh + c) = h;
                    const int64_t x = x0 + r;
                    if (save && x < X) *reinterpret_cast<float2*>(save + x * H + c) = h;
                }
            __syncthreads();
        }
        // ---- head (s, t) = h2 W3 + b3 and the affine coupling: 32 columns (16 pairs) per warp ----
        {
            const int n0 = 32 * half;
            float acc[4][4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const float b0 = bb3[n0 + 8 * nt + 2 * t], b1 = bb3[n0 + 8 * nt + 2 * t + 1];
                acc[nt][0] = b0; acc[nt][1] = b1; acc[nt][2] = b0; acc[nt][3] = b1;
            }
            mma_tile<4>(hs, ldh, H / 16, w3h, w3l, md.ldw3, n0, acc);
            float ls[2] = {0.f, 0.f};
            float ybv[4][2];                          // the b half's inputs, loaded together
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int j = (n0 + 8 * nt + 2 * t) >> 1;
                    const int64_t x = x0 + r0 + 8 * hh;
                    ybv[nt][hh] = (j < J && x < X) ? y[x * D + ib[j]] : 0.f;
                }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = r0 + 8 * hh, j = (n0 + 8 * nt + 2 * t) >> 1;
                    const int64_t x = x0 + r;
                    if (j >= J || x >= X) continue;
                    const float sv_s = kKappa * tanhf(acc[nt][2 * hh] / kKappa);
                    const float to = acc[nt][2 * hh + 1];
                    const int bi = ib[j];
                    const float yb = ybv[nt][hh];
                    const float out = (dir > 0) ? fmaf(yb, __expf(sv_s), to) : (yb - to) * __expf(-sv_s);
                    y[x * D + bi] = out;
                    ls[hh] += sv_s;
                    if (sv.s) { sv.s[x * J + j] = sv_s; sv.yb[x * J + j] = out; }
                }
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                ls[hh] += __shfl_xor_sync(0xffffffffu, ls[hh], 1);
                ls[hh] += __shfl_xor_sync(0xffffffffu, ls[hh], 2);
            }
            if (t == 0) { rsum[half * kTileS + r0] = ls[0]; rsum[half * kTileS + r0 + 8] = ls[1]; }
            __syncthreads();
            if (threadIdx.x < kTileS) {
                const int64_t x = x0 + threadIdx.x;
                if (x < X) {
                    const float s = rsum[threadIdx.x] + rsum[kTileS + threadIdx.x];
                    logdet[x] += (dir > 0) ? static_cast<double>(s) : -static_cast<double>(s);
                }
            }
        }
    }
}

// Back-propagation through one layer of the inverse direction, tiled like the forward pass: the
// coupling terms elementwise, then gz2 = (g_o W3^T) (1 - h2^2), gz1 = (gz2 W2^T) (1 - h1^2) and
// dL/dya = gz1 W1^T as shared-memory GEMMs against the transposed weights.
template <int HB>
__global__ void __launch_bounds__(kTileThreads) flow_tile_bwd_kernel(const LayerDev L, int64_t X,
                                                                     float* __restrict__ gy,
                                                                     const float* __restrict__ rt,
                                                                     const SaveDev sv, float* __restrict__ g_o,
                                                                     float* __restrict__ g_z2,
                                                                     float* __restrict__ g_z1) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D, O = 2 * J;
    const TileDims td(I, J, H, HB);
    const int Hp = td.Hp, Op = td.Op, Ip = td.Ip, ldo = td.ldo, ldh = td.ldh;
    float* w3t = fsm;                     // [Op][Hp]: row 2j + (0: s_j, 1: t_j) of W3^T
    float* w2t = w3t + Op * Hp;           // [Hp][Hp] = W2^T
    float* w1t = w2t + Hp * Hp;           // [Hp][Ip] = W1^T
    float* go = w1t + Hp * Ip;            // [64][ldo]
    float* gz = go + kTileS * ldo;        // [64][ldh]: gz2, then gz1
    int* ia = reinterpret_cast<int*>(gz + kTileS * ldh);   // idx_a [I], idx_b [J]
    int* ib = ia + I;
    for (int i = threadIdx.x; i < I + J; i += blockDim.x) ia[i] = i < I ? L.idx_a[i] : L.idx_b[i - I];
    // transposed copies: written along the shared-memory rows (a store across them would hit one
    // bank per warp), read across the source rows with eight loads in flight per thread
    block_copy(Op * Hp, [&](int i) { const int c = i / Hp, h = i - c * Hp, j = c >> 1;
                                     return (j < J && h < H) ? L.W3[h * O + ((c & 1) ? J + j : j)] : 0.f; },
               [&](int i, float v) { w3t[i] = v; });
    block_copy(Hp * Hp, [&](int i) { const int m = i / Hp, h = i - m * Hp;
                                     return (m < H && h < H) ? L.W2[h * H + m] : 0.f; },
               [&](int i, float v) { w2t[i] = v; });
    block_copy(Hp * Ip, [&](int i) { const int h = i / Ip, a = i - h * Ip;
                                     return (h < H && a < I) ? L.W1[a * H + h] : 0.f; },
               [&](int i, float v) { w1t[i] = v; });
    const int sg = threadIdx.x >> 4, cg = threadIdx.x & 15;
    const int OH = Op >> 1;
    const int64_t ntiles = (X + kTileS - 1) / kTileS;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t x0 = t * kTileS;
        __syncthreads();
        // ---- coupling: dL/d(s, t) per pair, dL/dyb' in place ----
        for (int i = threadIdx.x; i < kTileS * OH; i += blockDim.x) {
            const int s = i / OH, j = i - s * OH;
            const int64_t x = x0 + s;
            float gos = 0.f, gt = 0.f;
            if (j < J && x < X) {
                const int bi = ib[j];
                const float sj = sv.s[x * J + j], yb = sv.yb[x * J + j];
                const float gyb = gy[x * D + bi];
                const float es = __expf(-sj);
                gos = (-gyb * yb + rt[x]) * (1.0f - (sj / kKappa) * (sj / kKappa));
                gt = -gyb * es;
                gy[x * D + bi] = gyb * es;
                g_o[x * O + j] = gos;
                g_o[x * O + J + j] = gt;
            }
            go[s * ldo + 2 * j] = gos;
            go[s * ldo + 2 * j + 1] = gt;
        }
        __syncthreads();
        float acc[4][4 * HB];
        // ---- gz2 ----
        tile_init<HB>(acc, nullptr, 0, cg);
        tile_gemm<HB>(go, ldo, Op, w3t, Hp, 0, sg, cg, acc);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t x = x0 + 4 * sg + r;
#pragma unroll
            for (int u = 0; u < HB; ++u) {
                const int c = 4 * cg + 64 * u;
                const bool ok = x < X && c < H;
                const float4 h = ok ? *reinterpret_cast<const float4*>(sv.h2 + x * H + c) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 v = make_float4(acc[r][4 * u] * (1.f - h.x * h.x), acc[r][4 * u + 1] * (1.f - h.y * h.y),
                                             acc[r][4 * u + 2] * (1.f - h.z * h.z), acc[r][4 * u + 3] * (1.f - h.w * h.w));
                *reinterpret_cast<float4*>(gz + (4 * sg + r) * ldh + c) = v;
                if (ok) *reinterpret_cast<float4*>(g_z2 + x * H + c) = v;
            }
        }
        __syncthreads();
        // ---- gz1 ----
        tile_init<HB>(acc, nullptr, 0, cg);
        tile_gemm<HB>(gz, ldh, Hp, w2t, Hp, 0, sg, cg, acc);
        __syncthreads();                  // every read of gz2 is done
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t x = x0 + 4 * sg + r;
#pragma unroll
            for (int u = 0; u < HB; ++u) {
                const int c = 4 * cg + 64 * u;
                const bool ok = x < X && c < H;
                const float4 h = ok ? *reinterpret_cast<const float4*>(sv.h1 + x * H + c) : make_float4(0.f, 0.f, 0.f, 0.f);
                const float4 v = make_float4(acc[r][4 * u] * (1.f - h.x * h.x), acc[r][4 * u + 1] * (1.f - h.y * h.y),
                                             acc[r][4 * u + 2] * (1.f - h.z * h.z), acc[r][4 * u + 3] * (1.f - h.w * h.w));
                *reinterpret_cast<float4*>(gz + (4 * sg + r) * ldh + c) = v;
                if (ok) *reinterpret_cast<float4*>(g_z1 + x * H + c) = v;
            }
        }
        __syncthreads();
        // ---- dL/dya = gz1 W1^T, added at the a half ----
        for (int cb = 0; cb < Ip; cb += 64) {
            float o[4][4];
            tile_init<1>(o, nullptr, cb, cg);
            tile_gemm<1>(gz, ldh, Hp, w1t, Ip, cb, sg, cg, o);
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int64_t x = x0 + 4 * sg + r;
                if (x >= X) continue;
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int a = cb + 4 * cg + v;
                    if (a < I) gy[x * D + ia[a]] += o[r][v];
                }
            }
        }
    }
}

// Back-propagation through one layer on the tensor cores (the shapes of flow_tile_fwd_mma_kernel):
// the coupling terms elementwise as in flow_tile_bwd_kernel, then gz2 = (g_o W3^T)(1 - h2^2),
// gz1 = (gz2 W2^T)(1 - h1^2) and dL/dya = gz1 W1^T by the BF16 hi/lo MMAs of mma_tile.
struct MmaBwdDims {
    int ldw3, ldw2, ldw1, ldo, ldh;
    __host__ __device__ MmaBwdDims() : ldw3(32 + 4), ldw2(kMmaH / 2 + 4), ldw1(kMmaH / 2 + 4), ldo(64 + 8), ldh(kMmaH + 8) {}
    __host__ __device__ int words(int I, int J) const {
        return 2 * (kMmaH * ldw3 + kMmaH * ldw2 + 64 * ldw1) + kTileS * (ldo + ldh) + ((I + J + 3) / 4) * 4;
    }
};

__global__ void __launch_bounds__(kTileThreads) flow_tile_bwd_mma_kernel(const LayerDev L, int64_t X,
                                                                         float* __restrict__ gy,
                                                                         const float* __restrict__ rt,
                                                                         const SaveDev sv, float* __restrict__ g_o,
                                                                         float* __restrict__ g_z2,
                                                                         float* __restrict__ g_z1) {
    extern __shared__ __align__(16) uint32_t msm[];
    const int I = L.I, J = L.J, D = L.D, O = 2 * J, H = kMmaH;
    const MmaBwdDims md;
    const int ldo = md.ldo, ldh = md.ldh;
    uint32_t* w3h = msm;                        // B of gz2: [h][j] = (W3[h][j] (s), W3[h][J + j] (t))
    uint32_t* w3l = w3h + H * md.ldw3;
    uint32_t* w2h = w3l + H * md.ldw3;          // B of gz1: [h][m pairs] = W2[h][2m], W2[h][2m + 1]
    uint32_t* w2l = w2h + H * md.ldw2;
    uint32_t* w1h = w2l + H * md.ldw2;          // B of dya: [a][h pairs] = W1[a][2h], W1[a][2h + 1]
    uint32_t* w1l = w1h + 64 * md.ldw1;
    float* go = reinterpret_cast<float*>(w1l + 64 * md.ldw1);   // [64][ldo]: (g_s, g_t) of pair j at 2j, 2j + 1
    float* gz = go + kTileS * ldo;              // [64][ldh]: gz2, then gz1
    int* ia = reinterpret_cast<int*>(gz + kTileS * ldh);
    int* ib = ia + I;
    for (int i = threadIdx.x; i < I + J; i += blockDim.x) ia[i] = i < I ? L.idx_a[i] : L.idx_b[i - I];
    // stage_wt(get(k, n)) packs B[k][n] pairs along k into row n
    stage_wt<false>(H, 32, md.ldw3, w3h, w3l, [&](int k, int n) {
        const int j = k >> 1;
        return j < J ? L.W3[n * O + ((k & 1) ? J + j : j)] : 0.f;
    });
    stage_wt<false>(H, H / 2, md.ldw2, w2h, w2l, [&](int k, int n) { return L.W2[n * H + k]; });
    stage_wt<false>(64, H / 2, md.ldw1, w1h, w1l, [&](int k, int n) { return n < I ? L.W1[n * H + k] : 0.f; });
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int r0 = 16 * (warp & 3) + g;
    const int half = warp >> 2;
    const int64_t ntiles = (X + kTileS - 1) / kTileS;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t x0 = tile * kTileS;
        __syncthreads();
        // ---- coupling: dL/d(s, t) per pair, dL/dyb' in place (each thread's eight pairs' loads
        //      issued together) ----
        {
            float sj[8], ybv[8], gyb[8], rx[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = threadIdx.x + u * blockDim.x, s = i >> 5, j = i & 31;
                const int64_t x = x0 + s;
                const bool ok = j < J && x < X;
                sj[u] = ok ? sv.s[x * J + j] : 0.f;
                ybv[u] = ok ? sv.yb[x * J + j] : 0.f;
                gyb[u] = ok ? gy[x * D + ib[j]] : 0.f;
                rx[u] = ok ? rt[x] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int i = threadIdx.x + u * blockDim.x, s = i >> 5, j = i & 31;
                const int64_t x = x0 + s;
                float gos = 0.f, gt = 0.f;
                if (j < J && x < X) {
                    const float es = __expf(-sj[u]);
                    gos = (-gyb[u] * ybv[u] + rx[u]) * (1.0f - (sj[u] / kKappa) * (sj[u] / kKappa));
                    gt = -gyb[u] * es;
                    gy[x * D + ib[j]] = gyb[u] * es;
                    g_o[x * O + j] = gos;
                    g_o[x * O + J + j] = gt;
                }
                go[s * ldo + 2 * j] = gos;
                go[s * ldo + 2 * j + 1] = gt;
            }
        }
        static_assert(kTileS * 32 == 8 * kTileThreads, "the coupling's eight pairs per thread");
        __syncthreads();
        // ---- gz2, then gz1: 64 columns per warp ----
        for (int stage = 0; stage < 2; ++stage) {
            const int n0 = 64 * half;
            float acc[8][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
            if (stage == 0) mma_tile<8>(go, ldo, 4, w3h, w3l, md.ldw3, n0, acc);
            else mma_tile<8>(gz, ldh, H / 16, w2h, w2l, md.ldw2, n0, acc);
            if (stage == 1) __syncthreads();      // every read of gz2 is done
            const float* hsave = stage == 0 ? sv.h2 : sv.h1;
            float* gout = stage == 0 ? g_z2 : g_z1;
            float2 hv[8][2];                          // the saved activations, loaded together
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int64_t x = x0 + r0 + 8 * hh;
                    hv[nt][hh] = x < X ? *reinterpret_cast<const float2*>(hsave + x * H + n0 + 8 * nt + 2 * t)
                                       : make_float2(0.f, 0.f);
                }
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int r = r0 + 8 * hh, c = n0 + 8 * nt + 2 * t;
                    const int64_t x = x0 + r;
                    const bool ok = x < X;
                    const float2 h = hv[nt][hh];
                    const float2 v = make_float2(acc[nt][2 * hh] * (1.f - h.x * h.x), acc[nt][2 * hh + 1] * (1.f - h.y * h.y));
                    *reinterpret_cast<float2*>(gz + r * ldh + c) = v;
                    if (ok) *reinterpret_cast<float2*>(gout + x * H + c) = v;
                }
            __syncthreads();
        }
        // ---- dL/dya = gz1 W1^T, added at the a half: 32 columns per warp ----
        {
            const int n0 = 32 * half;
            float acc[4][4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) acc[nt][e] = 0.f;
            mma_tile<4>(gz, ldh, H / 16, w1h, w1l, md.ldw1, n0, acc);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int r = r0 + 8 * (e >> 1), a = n0 + 8 * nt + 2 * t + (e & 1);
                    const int64_t x = x0 + r;
                    if (a < I && x < X) gy[x * D + ia[a]] += acc[nt][e];
                }
        }
    }
}

// C[M][N] (+)= sum_x A[x][M] B[x][N] (the weight gradients: the batch is the reduction): a block
// computes a 64 x 64 tile of C over one contiguous split of the batch, 256 threads with 4 x 4
// outputs each from register-blocked outer products (two 128-bit shared loads per 16 FMAs); the
// splits' partials are added in a fixed order by gemm_tn_reduce, so the result is deterministic.
constexpr int kGBM = 64, kGBN = 64, kGBK = 32, kGPad = 4;
// batch rows per split of the weight-gradient GEMM (at most 64 splits); a build-time tunable
#ifndef PBR_GEMM_ROWS_PER_SPLIT
#define PBR_GEMM_ROWS_PER_SPLIT 256
#endif
constexpr int kGemmRowsPerSplit = PBR_GEMM_ROWS_PER_SPLIT;
static_assert(kGBK * kGBM == 8 * 256 && kGBM == 64 && kGBN == 64, "gemm_tn_partial's staging: 8 elements per thread");

// TF32 hi and lo parts of x (round to nearest), as the 32-bit patterns mma.sync takes
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(x));
    const float r = x - __uint_as_float(hi);
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(r));
}

// D (16 x 8, FP32) += A (16 x 8) B (8 x 8), TF32 operands
__device__ __forceinline__ void mma_tf32_1688(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Weight-gradient GEMM C = A^T B over the batch (A [X][M], B [X][N] row-major), split over the
// batch: each block stages kGBK batch rows of a 64 x 64 output tile in shared memory and its 8
// warps multiply them on the tensor cores (mma.sync m16n8k8, TF32 hi/lo split of both operands,
// three MMAs per step: about FP32 accuracy); warp w owns rows 16 (w % 4) .. + 15 and columns
// 32 (w / 4) .. + 31 of the tile.
__global__ void __launch_bounds__(256, 2) gemm_tn_partial(const float* __restrict__ A, const float* __restrict__ B,
                                                       int64_t X, int M, int N, int64_t chunk, int with_colsum,
                                                       float* __restrict__ part) {
    __shared__ __align__(16) float sa[kGBK][kGBM + kGPad];
    __shared__ __align__(16) float sb[kGBK][kGBN + kGPad];
    // column sums of B ride along in the first row of blocks: thread (tx, ty) adds rows 2 ty and
    // 2 ty + 1 of each staged tile for its four columns; the 16 partials are added in ty order
    const bool colsum = with_colsum && blockIdx.x == 0;
    float bs[4] = {0.f, 0.f, 0.f, 0.f};
    const int tm = blockIdx.x * kGBM, tn = blockIdx.y * kGBN, split = blockIdx.z;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int wm = 16 * (warp & 3), wn = 32 * (warp >> 2);
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    const int64_t x0 = split * chunk, x1 = min(X, x0 + chunk);
    // the next kGBK rows of both operands are loaded into registers while the current ones are
    // multiplied (8 elements of each per thread: element i = threadIdx.x + 256 u of the 32 x 64
    // tile), then stored after the barrier
    float na[8], nb[8];
    auto fetch = [&](int64_t xb) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = threadIdx.x + 256 * u, r = i >> 6, c = i & 63;
            const int64_t xx = xb + r;
            const bool ok = xx < x1;
            na[u] = (ok && tm + c < M) ? A[xx * M + tm + c] : 0.f;
            nb[u] = (ok && tn + c < N) ? B[xx * N + tn + c] : 0.f;
        }
    };
    if (x0 < x1) fetch(x0);
    for (int64_t xb = x0; xb < x1; xb += kGBK) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int i = threadIdx.x + 256 * u, r = i >> 6, c = i & 63;
            sa[r][c] = na[u];
            sb[r][c] = nb[u];
        }
        __syncthreads();
        if (xb + kGBK < x1) fetch(xb + kGBK);
        if (colsum) {
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
                const float4 v = *reinterpret_cast<const float4*>(&sb[2 * ty + kk][tx * 4]);
                bs[0] += v.x; bs[1] += v.y; bs[2] += v.z; bs[3] += v.w;
            }
        }
#pragma unroll
        for (int k0 = 0; k0 < kGBK; k0 += 8) {
            // A^T fragment: rows = output rows m, columns = batch rows k
            uint32_t ah[4], al[4];
            split_tf32(sa[k0 + t][wm + g], ah[0], al[0]);
            split_tf32(sa[k0 + t][wm + g + 8], ah[1], al[1]);
            split_tf32(sa[k0 + t + 4][wm + g], ah[2], al[2]);
            split_tf32(sa[k0 + t + 4][wm + g + 8], ah[3], al[3]);
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                uint32_t bh0, bl0, bh1, bl1;
                split_tf32(sb[k0 + t][wn + 8 * nt + g], bh0, bl0);
                split_tf32(sb[k0 + t + 4][wn + 8 * nt + g], bh1, bl1);
                mma_tf32_1688(acc[nt], ah, bh0, bh1);
                mma_tf32_1688(acc[nt], ah, bl0, bl1);
                mma_tf32_1688(acc[nt], al, bh0, bh1);
            }
        }
        __syncthreads();
    }
    // partials: [split][M + 1][N], row M = the column sums; fragment element (row g / g + 8,
    // columns 2 t, 2 t + 1) of each 16 x 8 tile
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int m = tm + wm + g + 8 * (e >> 1), n = tn + wn + 8 * nt + 2 * t + (e & 1);
            if (m < M && n < N) part[(static_cast<int64_t>(split) * (M + 1) + m) * N + n] = acc[nt][e];
        }
    if (colsum) {                                  // block-uniform
#pragma unroll
        for (int j = 0; j < 4; ++j) sa[ty][tx * 4 + j] = bs[j];    // sa is free after the last tile
        __syncthreads();
        if (ty == 0) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float tt = 0.f;
                for (int r = 0; r < 16; ++r) tt += sa[r][tx * 4 + j];
                const int n = tn + tx * 4 + j;
                if (n < N) part[(static_cast<int64_t>(split) * (M + 1) + M) * N + n] = tt;
            }
        }
    }
}

// partials [splits][M + 1][N] added in split order: rows < M into C, row M into colsum (if any)
// C = beta C + the sum of the splits' partial products (and colsum = the sum of their column-sum
// rows).  A block takes 32 consecutive outputs; its warp u sums the splits s = u (mod 8) in
// increasing s, and the eight warp sums are added in u order: a fixed order, the same as one
// thread per output keeping eight running sums, but with 8 loads per thread instead of 64 in
// sequence (the one-thread form held 16-65 blocks at the training shapes and waited on its loads).
__global__ void __launch_bounds__(256) gemm_tn_reduce(const float* __restrict__ part, int splits, int M, int N,
                                                      float beta, float* __restrict__ C, float* __restrict__ colsum) {
    __shared__ float red[8][32];
    const int MN = M * N, total = colsum ? MN + N : MN;
    const int64_t stride = MN + N;
    const int lane = threadIdx.x & 31, u = threadIdx.x >> 5;
    for (int i0 = blockIdx.x * 32; i0 < total; i0 += gridDim.x * 32) {
        const int i = i0 + lane;
        float a = 0.f;
        if (i < total) {
#pragma unroll 8
            for (int s = u; s < splits; s += 8) a += part[static_cast<int64_t>(s) * stride + i];
        }
        red[u][lane] = a;
        __syncthreads();
        if (u == 0 && i < total) {
            float acc = 0.f;
#pragma unroll
            for (int v = 0; v < 8; ++v) acc += red[v][lane];
            if (i < MN) C[i] = (beta == 0.f) ? acc : beta * C[i] + acc;   // beta == 0: C may hold garbage
            else colsum[i - MN] = acc;
        }
        __syncthreads();
    }
}

// out[n] = sum_x B[x][n] (fixed order: thread per column, sequential over the batch in 4 lanes)
__global__ void colsum_kernel(const float* __restrict__ B, int64_t X, int N, float* __restrict__ out) {
    const int n = blockIdx.x;
    float acc = 0.f;
    for (int64_t x = threadIdx.x; x < X; x += blockDim.x) acc += B[x * N + n];
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o >= 1; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = red[0];
}

// Base mixture: lse[x] = log sum_a exp(log_pi_a - |y0 - mu_a|^2/2), rgam[x][a] = rt_x gamma_xa,
// gy[x] = rt_x sum_a gamma_xa (y0 - mu_a), lossterm[x] = -rt_x (lse + ld).
__global__ void flow_base_kernel(const float* __restrict__ y0, const double* __restrict__ ld, int64_t X, int D,
                                 int A, const float* __restrict__ mu, const float* __restrict__ log_pi,
                                 const float* __restrict__ rt, float* __restrict__ gy, float* __restrict__ rgam,
                                 double* __restrict__ lossterm, double* __restrict__ lse_out) {
    for (int64_t x = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; x < X;
         x += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float* yx = y0 + x * D;
        float e[16];
        float mx = -INFINITY;
        for (int a = 0; a < A; ++a) {
            float d2 = 0.f;
            for (int k = 0; k < D; ++k) { const float d = yx[k] - mu[a * D + k]; d2 = fmaf(d, d, d2); }
            e[a] = log_pi[a] - 0.5f * d2;
            mx = fmaxf(mx, e[a]);
        }
        float den = 0.f;
        for (int a = 0; a < A; ++a) { e[a] = __expf(e[a] - mx); den += e[a]; }
        // den is in [1, A]: its FP32 log is exact to ~1e-7 absolute, the scale of mx in FP64
        const double lse = static_cast<double>(mx) + static_cast<double>(logf(den));
        const float w = rt ? rt[x] : 0.f;
        for (int a = 0; a < A; ++a) {
            e[a] /= den;
            if (rgam) rgam[x * A + a] = w * e[a];
        }
        if (gy) {
            for (int k = 0; k < D; ++k) {
                float g = 0.f;
                for (int a = 0; a < A; ++a) g = fmaf(e[a], yx[k] - mu[a * D + k], g);
                gy[x * D + k] = w * g;
            }
        }
        if (lossterm) lossterm[x] = -static_cast<double>(w) * (lse + ld[x]);
        if (lse_out) lse_out[x] = lse;
    }
}

// Proposal density of x = F(q) in the scale of x's PIMC outputs:
//   s_q[x] = exp(log rho(q) - logdet_f - log_scale(x)),
//   log rho(q) = logsumexp_a (logC_a - |y - mu_a|^2/2) - U/2
__global__ void flow_weights_kernel(const double* __restrict__ lse_y, const double* __restrict__ U,
                                    const double* __restrict__ logdet, const double* __restrict__ log_scale_x,
                                    int64_t X, double* __restrict__ s_q) {
    for (int64_t x = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; x < X;
         x += static_cast<int64_t>(gridDim.x) * blockDim.x)
        s_q[x] = pbr::exp_out_fp32(lse_y[x] - 0.5 * U[x] - logdet[x] - log_scale_x[x]);
}

__global__ void adam_count_kernel(int32_t* step) { *step += 1; }

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                            const int32_t* __restrict__ step) {
    const float t = static_cast<float>(*step);
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

int grid_for(int64_t n, int threads) {
    const int64_t g = (n + threads - 1) / threads;
    const int cap = sm_count() * 16;
    return static_cast<int>(g < cap ? (g > 0 ? g : 1) : cap);
}

int status() { return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA; }

int layer_smem_fwd(const pbr_flow_layer* l) {
    return static_cast<int>(sizeof(float)) *
           (l->I * l->H + l->H * l->H + l->H * 2 * l->J + 2 * l->H + align_up_(2 * l->J, 4) +
            kFlowWarps * (align_up_(l->I, 4) + 2 * l->H));
}
int layer_smem_bwd(const pbr_flow_layer* l) {
    return static_cast<int>(sizeof(float)) *
           (l->H * align_up_(l->I, 32) + l->H * l->H + 2 * l->J * l->H +
            kFlowWarps * (align_up_(2 * l->J, 4) + 2 * l->H));
}

// hidden widths 32, 64, 128, 256: UPH = H / 32 units per lane
bool layer_ok(const pbr_flow_layer* l) {
    return l && l->D > 0 && l->I > 0 && l->J > 0 && (l->H == 32 || l->H == 64 || l->H == 128 || l->H == 256) &&
           l->I + l->J == l->D && l->idx_a &&
           l->idx_b && l->W1 && l->b1 && l->W2 && l->b2 && l->W3 && l->b3;
}

// Shared memory of the sample-tiled layer kernels, or 0 when they do not apply (H > 128, or the
// padded weights and tiles exceed a block's shared memory): the warp-per-sample kernels then run.
int tile_smem(const pbr_flow_layer* l, bool fwd) {
    if (l->H > 128) return 0;
    const TileDims td(l->I, l->J, l->H, l->H > 64 ? 2 : 1);
    const int64_t bytes = static_cast<int64_t>(sizeof(float)) *
                          (fwd ? td.fwd_floats(l->I, l->J) : td.bwd_floats(l->I, l->J));
    return bytes <= 227 * 1024 ? static_cast<int>(bytes) : 0;
}

// persistent grid: one block per resident slot, no more blocks than tiles; 0 when it cannot run
template <typename K>
int tile_grid(K kern, int bytes, int64_t X) {
    const int occ = resident_blocks(kern, kTileThreads, bytes);
    if (occ < 1) return 0;
    const int64_t tiles = (X + kTileS - 1) / kTileS;
    const int64_t cap = static_cast<int64_t>(sm_count()) * occ;
    return static_cast<int>(tiles < cap ? tiles : cap);
}

LayerDev to_dev(const pbr_flow_layer* l) {
    return LayerDev{l->D, l->I, l->J, l->H, l->idx_a, l->idx_b, l->W1, l->b1, l->W2, l->b2, l->W3, l->b3};
}

}  // namespace

extern "C" {

int pbr_flow_prepare(const float* q, int64_t X, int32_t N, int32_t P, int32_t nsel, const double* center,
                     const double* inv_sigma, const double* rho_csch, const double* rho_tanh2, float* y,
                     double* U, void* stream) {
    if (!q || !center || !inv_sigma || !rho_csch || !rho_tanh2 || !y || !U) return PBR_ERR_ARG;
    // slots beyond the cos/sin pairs (the alternating mode of an even ring) are not supported
    if (X < 0 || N < 1 || P < 3 || P > 4096 || nsel < 1 || nsel > 8 || nsel > 1 + 2 * ((P - 1) / 2))
        return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const int threads = 256;
    if (N > threads) return PBR_ERR_UNSUPPORTED;
    const int bytes = static_cast<int>(sizeof(double)) * threads +
                      static_cast<int>(sizeof(float)) * (nsel * P + N * nsel + 4 * N);
    if (resident_blocks(flow_prepare_kernel, threads, bytes) < 1) return PBR_ERR_UNSUPPORTED;
    const int64_t spb = threads / N;
    flow_prepare_kernel<<<grid_for((X + spb - 1) / spb * threads, threads), threads, bytes,
                          static_cast<cudaStream_t>(stream)>>>(q, X, N, P, nsel, center, inv_sigma, rho_csch,
                                                               rho_tanh2, y, U);
    return status();
}

int pbr_flow_apply(const float* q, const float* y, const float* y_new, int64_t X, int32_t N, int32_t P,
                   int32_t nsel, const double* sigma, float* x, void* stream) {
    if (!q || !y || !y_new || !sigma || !x || X < 0 || N < 1 || P < 3 || P > 4096 || nsel < 1 || nsel > 8 ||
        nsel > 1 + 2 * ((P - 1) / 2))
        return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const int bytes = static_cast<int>(sizeof(float)) * (nsel * P + N * nsel);
    if (resident_blocks(flow_apply_kernel, 256, bytes) < 1) return PBR_ERR_UNSUPPORTED;
    flow_apply_kernel<<<grid_for((X * N + kApplyRows - 1) / kApplyRows * 32, 256), 256, bytes,
                        static_cast<cudaStream_t>(stream)>>>(
        q, y, y_new, X, N, P, nsel, sigma, x);
    return status();
}

int pbr_flow_layer_forward(const pbr_flow_layer* layer, int32_t direction, int64_t X, float* y,
                           double* logdet, const pbr_flow_save* save, void* stream) {
    if (!layer_ok(layer) || !y || !logdet || X < 0 || (direction != 1 && direction != -1)) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    SaveDev sv{nullptr, nullptr, nullptr, nullptr, nullptr};
    if (save) {
        if (!save->ya || !save->h1 || !save->h2 || !save->s || !save->yb) return PBR_ERR_ARG;
        sv = SaveDev{save->ya, save->h1, save->h2, save->s, save->yb};
    }
    // the training direction with saves: the tensor-core tile kernel where its shapes apply
    if (save && layer->H == kMmaH && layer->I <= 64 && 2 * layer->J <= 64) {
        const int mb = static_cast<int>(sizeof(uint32_t)) * MmaDims(layer->I, layer->J).fwd_words(layer->I, layer->J);
        if (mb <= 227 * 1024) {
            const int grid = tile_grid(flow_tile_fwd_mma_kernel, mb, X);
            if (grid >= 1) {
                flow_tile_fwd_mma_kernel<<<grid, kTileThreads, mb, static_cast<cudaStream_t>(stream)>>>(
                    to_dev(layer), direction, X, y, logdet, sv);
                return status();
            }
        }
    }
    const int tb = tile_smem(layer, true);
    if (tb > 0) {
        auto run = [&](auto kern) -> int {
            const int grid = tile_grid(kern, tb, X);
            if (grid < 1) return PBR_ERR_UNSUPPORTED;
            kern<<<grid, kTileThreads, tb, static_cast<cudaStream_t>(stream)>>>(to_dev(layer), direction, X, y,
                                                                                 logdet, sv);
            return status();
        };
        return layer->H > 64 ? run(flow_tile_fwd_kernel<2>) : run(flow_tile_fwd_kernel<1>);
    }
    const int bytes = layer_smem_fwd(layer);
    if (bytes > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    auto go = [&](auto kern) -> int {
        const int occ = resident_blocks(kern, kFlowWarps * 32, bytes);
        if (occ < 1) return PBR_ERR_UNSUPPORTED;
        const int64_t blocks = (X + kFlowWarps - 1) / kFlowWarps;
        const int cap = sm_count() * occ;
        kern<<<static_cast<int>(blocks < cap ? blocks : cap), kFlowWarps * 32, bytes,
               static_cast<cudaStream_t>(stream)>>>(to_dev(layer), direction, X, y, logdet, sv);
        return status();
    };
    switch (layer->H) {
        case 32: return go(flow_layer_fwd_kernel<1>);
        case 64: return go(flow_layer_fwd_kernel<2>);
        case 128: return go(flow_layer_fwd_kernel<4>);
        default: return go(flow_layer_fwd_kernel<8>);
    }
}

int pbr_flow_layer_backward(const pbr_flow_layer* layer, int64_t X, float* gy, const float* rt,
                            const pbr_flow_save* save, float* g_o, float* g_z2, float* g_z1, void* stream) {
    if (!layer_ok(layer) || !gy || !rt || !save || !g_o || !g_z2 || !g_z1 || X < 0) return PBR_ERR_ARG;
    if (!save->h1 || !save->h2 || !save->s || !save->yb) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const SaveDev sv{save->ya, save->h1, save->h2, save->s, save->yb};
    if (layer->H == kMmaH && layer->I <= 64 && 2 * layer->J <= 64) {
        const int mb = static_cast<int>(sizeof(uint32_t)) * MmaBwdDims().words(layer->I, layer->J);
        if (mb <= 227 * 1024) {
            const int grid = tile_grid(flow_tile_bwd_mma_kernel, mb, X);
            if (grid >= 1) {
                flow_tile_bwd_mma_kernel<<<grid, kTileThreads, mb, static_cast<cudaStream_t>(stream)>>>(
                    to_dev(layer), X, gy, rt, sv, g_o, g_z2, g_z1);
                return status();
            }
        }
    }
    const int tb = tile_smem(layer, false);
    if (tb > 0) {
        auto run = [&](auto kern) -> int {
            const int grid = tile_grid(kern, tb, X);
            if (grid < 1) return PBR_ERR_UNSUPPORTED;
            kern<<<grid, kTileThreads, tb, static_cast<cudaStream_t>(stream)>>>(to_dev(layer), X, gy, rt, sv, g_o,
                                                                                 g_z2, g_z1);
            return status();
        };
        return layer->H > 64 ? run(flow_tile_bwd_kernel<2>) : run(flow_tile_bwd_kernel<1>);
    }
    const int bytes = layer_smem_bwd(layer);
    if (bytes > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    auto go = [&](auto kern) -> int {
        const int occ = resident_blocks(kern, kFlowWarps * 32, bytes);
        if (occ < 1) return PBR_ERR_UNSUPPORTED;
        const int64_t blocks = (X + kFlowWarps - 1) / kFlowWarps;
        const int cap = sm_count() * occ;
        kern<<<static_cast<int>(blocks < cap ? blocks : cap), kFlowWarps * 32, bytes,
               static_cast<cudaStream_t>(stream)>>>(to_dev(layer), X, gy, rt, sv, g_o, g_z2, g_z1);
        return status();
    };
    switch (layer->H) {
        case 32: return go(flow_layer_bwd_kernel<1>);
        case 64: return go(flow_layer_bwd_kernel<2>);
        case 128: return go(flow_layer_bwd_kernel<4>);
        default: return go(flow_layer_bwd_kernel<8>);
    }
}

int64_t pbr_gemm_tn_scratch(int64_t X, int32_t M, int32_t N) {
    const int64_t s = X / kGemmRowsPerSplit;
    const int64_t splits = s < 1 ? 1 : (s < 64 ? s : 64);
    return splits * (static_cast<int64_t>(M) + 1) * N;
}

int pbr_gemm_tn_acc(const float* A, const float* B, int64_t X, int32_t M, int32_t N, float beta, float* C,
                    float* colsum, float* scratch, void* stream) {
    if (!A || !B || !C || !scratch || X < 1 || M < 1 || N < 1) return PBR_ERR_ARG;
    const int64_t splits = pbr_gemm_tn_scratch(X, M, N) / ((static_cast<int64_t>(M) + 1) * N);
    const int64_t chunk = (X + splits - 1) / splits;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grid((M + kGBM - 1) / kGBM, (N + kGBN - 1) / kGBN, static_cast<unsigned>(splits));
    gemm_tn_partial<<<grid, 256, 0, st>>>(A, B, X, M, N, chunk, colsum ? 1 : 0, scratch);
    const int64_t outs = (static_cast<int64_t>(M) + 1) * N;
    gemm_tn_reduce<<<static_cast<int>(std::min<int64_t>((outs + 31) / 32, 8192)), 256, 0, st>>>(
        scratch, static_cast<int>(splits), M, N, beta, C, colsum);
    return status();
}

int pbr_colsum(const float* B, int64_t X, int32_t N, float* out, void* stream) {
    if (!B || !out || X < 1 || N < 1) return PBR_ERR_ARG;
    colsum_kernel<<<N, 256, 0, static_cast<cudaStream_t>(stream)>>>(B, X, N, out);
    return status();
}

int pbr_flow_base(const float* y0, const double* ld, int64_t X, int32_t D, int32_t A, const float* mu,
                  const float* log_pi, const float* rt, float* gy, float* rgam, double* lossterm,
                  double* lse, void* stream) {
    if (!y0 || !mu || !log_pi || X < 0 || D < 1 || A < 1 || A > 16) return PBR_ERR_ARG;
    if (lossterm && !ld) return PBR_ERR_ARG;
    if ((gy || rgam || lossterm) && !rt) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    flow_base_kernel<<<grid_for(X, 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(
        y0, ld, X, D, A, mu, log_pi, rt, gy, rgam, lossterm, lse);
    return status();
}

int pbr_flow_weights(const double* lse_y, const double* U, const double* logdet, const double* log_scale_x,
                     int64_t X, double* s_q, void* stream) {
    if (!lse_y || !U || !logdet || !log_scale_x || !s_q || X < 0) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    flow_weights_kernel<<<grid_for(X, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(lse_y, U, logdet,
                                                                                         log_scale_x, X, s_q);
    return status();
}

int pbr_adam(float* param, const float* grad, float* m, float* v, int64_t n, float lr, float beta1,
             float beta2, float eps, int32_t* step, void* stream) {
    if (!param || !grad || !m || !v || !step || n < 0) return PBR_ERR_ARG;
    if (n == 0) return PBR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    adam_count_kernel<<<1, 1, 0, st>>>(step);
    adam_kernel<<<grid_for(n, 256), 256, 0, st>>>(param, grad, m, v, n, lr, beta1, beta2, eps, step);
    return status();
}

}  // extern "C"
