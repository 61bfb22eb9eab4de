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
#include <cmath>

#include "pbr_common.cuh"

namespace {

constexpr int kFlowWarps = 4;
constexpr float kKappa = 2.0f;

inline int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// ---------------------------------------------------------------------------------------------
// prepare: y[x][j*nsel + s] = (sum_p B_ps (q_jp - c_j)) * inv_sigma[j*nsel + s],
//          U[x] = sum_j (q_j - c_j)^T Lambda_j (q_j - c_j) - sum |y|^2
// Lambda_j = 2 coth I - csch C evaluated as sum_p csch (dx)^2 + 2 tanh(tau w/2) x_p^2.
// One warp per (sample); lanes over beads.
// ---------------------------------------------------------------------------------------------
__global__ void flow_prepare_kernel(const float* __restrict__ q, int64_t X, int N, int P, int nsel,
                                    const double* __restrict__ center, const double* __restrict__ inv_sigma,
                                    const double* __restrict__ rho_csch, const double* __restrict__ rho_tanh2,
                                    float* __restrict__ y, double* __restrict__ U) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t gw = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp;
    const int64_t nw = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    const double inv_sqrt_p = 1.0 / sqrt(static_cast<double>(P));
    const double amp = sqrt(2.0 / P);
    for (int64_t x = gw; x < X; x += nw) {
        double quad_total = 0.0, ysq = 0.0;
        for (int j = 0; j < N; ++j) {
            const float* qj = q + (x * N + j) * static_cast<int64_t>(P);
            const double c = center[j];
            double quad = 0.0;
            double proj[8];
#pragma unroll
            for (int s = 0; s < 8; ++s) proj[s] = 0.0;
            for (int p = lane; p < P; p += 32) {
                const double xp = static_cast<double>(qj[p]) - c;
                const double xn = static_cast<double>(qj[(p + 1 == P) ? 0 : p + 1]) - c;
                const double d = xp - xn;
                quad += rho_csch[j] * d * d + 2.0 * rho_tanh2[j] * xp * xp;
#pragma unroll
                for (int s = 0; s < 8; ++s) {
                    if (s >= nsel) break;
                    double bv;
                    if (s == 0) {
                        bv = inv_sqrt_p;
                    } else {
                        const int k = (s + 1) / 2;
                        double sn, cs;
                        sincospi(2.0 * k * p / P, &sn, &cs);
                        bv = amp * ((s & 1) ? cs : sn);
                    }
                    proj[s] += bv * xp;
                }
            }
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) {
                quad += __shfl_xor_sync(0xffffffffu, quad, o);
#pragma unroll
                for (int s = 0; s < 8; ++s) proj[s] += __shfl_xor_sync(0xffffffffu, proj[s], o);
            }
            quad_total += quad;
#pragma unroll
            for (int s = 0; s < 8; ++s) {
                if (s >= nsel) break;
                const double v = proj[s] * inv_sigma[j * nsel + s];
                ysq += v * v;
                if (lane == 0) y[x * static_cast<int64_t>(N * nsel) + j * nsel + s] = static_cast<float>(v);
            }
        }
        if (lane == 0) U[x] = quad_total - ysq;
    }
}

// x = q + sum_{s < nsel} B_ps sigma_js (y'_js - y_js)
__global__ void flow_apply_kernel(const float* __restrict__ q, const float* __restrict__ y,
                                  const float* __restrict__ yn, int64_t X, int N, int P, int nsel,
                                  const double* __restrict__ sigma, float* __restrict__ xo) {
    const int64_t total = X * N * static_cast<int64_t>(P);
    const double inv_sqrt_p = 1.0 / sqrt(static_cast<double>(P));
    const double amp = sqrt(2.0 / P);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int p = static_cast<int>(i % P);
        const int64_t xj = i / P;
        const int j = static_cast<int>(xj % N);
        const int64_t x = xj / N;
        double acc = q[i];
        for (int s = 0; s < nsel; ++s) {
            double bv;
            if (s == 0) {
                bv = inv_sqrt_p;
            } else {
                const int k = (s + 1) / 2;
                double sn, cs;
                sincospi(2.0 * k * p / P, &sn, &cs);
                bv = amp * ((s & 1) ? cs : sn);
            }
            const int64_t yi = x * static_cast<int64_t>(N * nsel) + j * nsel + s;
            acc += bv * sigma[j * nsel + s] * (static_cast<double>(yn[yi]) - static_cast<double>(y[yi]));
        }
        xo[i] = static_cast<float>(acc);
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

__global__ void flow_layer_fwd_kernel(const LayerDev L, int dir, int64_t X, float* __restrict__ y,
                                      double* __restrict__ logdet, const SaveDev sv) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D, O = 2 * J;
    float* w1 = fsm;
    float* w2 = w1 + I * H;
    float* w3 = w2 + H * H;
    float* bb1 = w3 + H * O;
    float* bb2 = bb1 + H;
    float* bb3 = bb2 + H;
    float* wbuf = bb3 + O;
    for (int i = threadIdx.x; i < I * H; i += blockDim.x) w1[i] = L.W1[i];
    for (int i = threadIdx.x; i < H * H; i += blockDim.x) w2[i] = L.W2[i];
    for (int i = threadIdx.x; i < H * O; i += blockDim.x) w3[i] = L.W3[i];
    for (int i = threadIdx.x; i < H; i += blockDim.x) { bb1[i] = L.b1[i]; bb2[i] = L.b2[i]; }
    for (int i = threadIdx.x; i < O; i += blockDim.x) bb3[i] = L.b3[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* ya = wbuf + warp * (I + 2 * H);
    float* h1 = ya + I;
    float* h2 = h1 + H;
    const int64_t nw = static_cast<int64_t>(gridDim.x) * kFlowWarps;
    for (int64_t x = static_cast<int64_t>(blockIdx.x) * kFlowWarps + warp; x < X; x += nw) {
        float* yx = y + x * D;
        for (int i = lane; i < I; i += 32) ya[i] = yx[L.idx_a[i]];
        __syncwarp();
        for (int h = lane; h < H; h += 32) {
            float z = bb1[h];
            for (int i = 0; i < I; ++i) z = fmaf(ya[i], w1[i * H + h], z);
            h1[h] = tanhf(z);
        }
        __syncwarp();
        for (int h = lane; h < H; h += 32) {
            float z = bb2[h];
            for (int k = 0; k < H; ++k) z = fmaf(h1[k], w2[k * H + h], z);
            h2[h] = tanhf(z);
        }
        __syncwarp();
        float ssum = 0.0f;
        for (int j = lane; j < J; j += 32) {
            float os = bb3[j], ot = bb3[J + j];
            for (int k = 0; k < H; ++k) {
                const float hk = h2[k];
                os = fmaf(hk, w3[k * O + j], os);
                ot = fmaf(hk, w3[k * O + J + j], ot);
            }
            const float s = kKappa * tanhf(os / kKappa);
            const int bi = L.idx_b[j];
            const float yb = yx[bi];
            const float out = (dir > 0) ? fmaf(yb, __expf(s), ot) : (yb - ot) * __expf(-s);
            yx[bi] = out;
            ssum += s;
            if (sv.s) { sv.s[x * J + j] = s; sv.yb[x * J + j] = out; }
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
__global__ void flow_layer_bwd_kernel(const LayerDev L, int64_t X, float* __restrict__ gy,
                                      const float* __restrict__ rt, const SaveDev sv,
                                      float* __restrict__ g_o, float* __restrict__ g_z2,
                                      float* __restrict__ g_z1) {
    extern __shared__ __align__(16) float fsm[];
    const int I = L.I, J = L.J, H = L.H, D = L.D, O = 2 * J;
    float* w1t = fsm;                 // [H][I]
    float* w2t = w1t + H * I;         // [H][H]  (transposed)
    float* w3t = w2t + H * H;         // [O][H]
    float* wbuf = w3t + O * H;
    for (int i = threadIdx.x; i < I * H; i += blockDim.x) {
        const int r = i / H, c = i - r * H;
        w1t[c * I + r] = L.W1[i];
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
    float* go = wbuf + warp * (O + 2 * H);
    float* gz2 = go + O;
    float* gz1 = gz2 + H;
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
        for (int h = lane; h < H; h += 32) {
            float acc = 0.0f;
            for (int c = 0; c < O; ++c) acc = fmaf(go[c], w3t[c * H + h], acc);
            const float h2v = sv.h2[x * H + h];
            const float v = acc * (1.0f - h2v * h2v);
            gz2[h] = v;
            g_z2[x * H + h] = v;
        }
        __syncwarp();
        for (int h = lane; h < H; h += 32) {
            float acc = 0.0f;
            for (int m = 0; m < H; ++m) acc = fmaf(gz2[m], w2t[m * H + h], acc);
            const float h1v = sv.h1[x * H + h];
            const float v = acc * (1.0f - h1v * h1v);
            gz1[h] = v;
            g_z1[x * H + h] = v;
        }
        __syncwarp();
        for (int i = lane; i < I; i += 32) {
            float acc = 0.0f;
            for (int k = 0; k < H; ++k) acc = fmaf(gz1[k], w1t[k * I + i], acc);
            gx[L.idx_a[i]] += acc;
        }
        __syncwarp();
    }
}

// C[M][N] (+)= sum_x A[x][M] B[x][N]: block = 32 x 32 tile x one batch split; partials reduced in
// split order by gemm_tn_reduce.
constexpr int kTile = 32;
__global__ void gemm_tn_partial(const float* __restrict__ A, const float* __restrict__ B, int64_t X, int M,
                                int N, int64_t chunk, float* __restrict__ part) {
    __shared__ float sa[kTile][kTile + 1], sb[kTile][kTile + 1];
    const int tm = blockIdx.x * kTile, tn = blockIdx.y * kTile, split = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8 threads
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    const int64_t x0 = split * chunk, x1 = min(X, x0 + chunk);
    for (int64_t xb = x0; xb < x1; xb += kTile) {
        for (int r = ty; r < kTile; r += 8) {
            const int64_t xx = xb + r;
            sa[r][tx] = (xx < x1 && tm + tx < M) ? A[xx * M + tm + tx] : 0.f;
            sb[r][tx] = (xx < x1 && tn + tx < N) ? B[xx * N + tn + tx] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < kTile; ++r) {
            const float bv = sb[r][tx];
#pragma unroll
            for (int u = 0; u < 4; ++u) acc[u] = fmaf(sa[r][ty + 8 * u], bv, acc[u]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int m = tm + ty + 8 * u, n = tn + tx;
        if (m < M && n < N) part[(static_cast<int64_t>(split) * M + m) * N + n] = acc[u];
    }
}

__global__ void gemm_tn_reduce(const float* __restrict__ part, int splits, int MN, float beta,
                               float* __restrict__ C) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MN; i += gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int s = 0; s < splits; ++s) acc += part[static_cast<int64_t>(s) * MN + i];
        C[i] = (beta == 0.f) ? acc : beta * C[i] + acc;   // beta == 0: C may hold garbage
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
        const double lse = static_cast<double>(mx) + log(static_cast<double>(den));
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
        s_q[x] = exp(lse_y[x] - 0.5 * U[x] - logdet[x] - log_scale_x[x]);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
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
           (l->I * l->H + l->H * l->H + l->H * 2 * l->J + 2 * l->H + 2 * l->J + kFlowWarps * (l->I + 2 * l->H));
}
int layer_smem_bwd(const pbr_flow_layer* l) {
    return static_cast<int>(sizeof(float)) *
           (l->I * l->H + l->H * l->H + 2 * l->J * l->H + kFlowWarps * (2 * l->J + 2 * l->H));
}

bool layer_ok(const pbr_flow_layer* l) {
    return l && l->D > 0 && l->I > 0 && l->J > 0 && l->H > 0 && l->I + l->J == l->D && l->idx_a &&
           l->idx_b && l->W1 && l->b1 && l->W2 && l->b2 && l->W3 && l->b3;
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
    if (X < 0 || N < 1 || P < 3 || nsel < 1 || nsel > 8 || nsel > 1 + 2 * ((P - 1) / 2)) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const int threads = 128;
    flow_prepare_kernel<<<grid_for(X * 32, threads), threads, 0, static_cast<cudaStream_t>(stream)>>>(
        q, X, N, P, nsel, center, inv_sigma, rho_csch, rho_tanh2, y, U);
    return status();
}

int pbr_flow_apply(const float* q, const float* y, const float* y_new, int64_t X, int32_t N, int32_t P,
                   int32_t nsel, const double* sigma, float* x, void* stream) {
    if (!q || !y || !y_new || !sigma || !x || X < 0 || N < 1 || P < 3 || nsel < 1 || nsel > 8 ||
        nsel > 1 + 2 * ((P - 1) / 2))
        return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    flow_apply_kernel<<<grid_for(X * N * P, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
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
    const int bytes = layer_smem_fwd(layer);
    if (bytes > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    if (bytes > 48 * 1024 &&
        cudaFuncSetAttribute(flow_layer_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
        return PBR_ERR_UNSUPPORTED;
    const int64_t blocks = (X + kFlowWarps - 1) / kFlowWarps;
    const int grid = static_cast<int>(blocks < sm_count() * 2 ? blocks : sm_count() * 2);
    flow_layer_fwd_kernel<<<grid, kFlowWarps * 32, bytes, static_cast<cudaStream_t>(stream)>>>(
        to_dev(layer), direction, X, y, logdet, sv);
    return status();
}

int pbr_flow_layer_backward(const pbr_flow_layer* layer, int64_t X, float* gy, const float* rt,
                            const pbr_flow_save* save, float* g_o, float* g_z2, float* g_z1, void* stream) {
    if (!layer_ok(layer) || !gy || !rt || !save || !g_o || !g_z2 || !g_z1 || X < 0) return PBR_ERR_ARG;
    if (!save->h1 || !save->h2 || !save->s || !save->yb) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const int bytes = layer_smem_bwd(layer);
    if (bytes > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    if (bytes > 48 * 1024 &&
        cudaFuncSetAttribute(flow_layer_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
        return PBR_ERR_UNSUPPORTED;
    const SaveDev sv{save->ya, save->h1, save->h2, save->s, save->yb};
    const int64_t blocks = (X + kFlowWarps - 1) / kFlowWarps;
    const int grid = static_cast<int>(blocks < sm_count() * 2 ? blocks : sm_count() * 2);
    flow_layer_bwd_kernel<<<grid, kFlowWarps * 32, bytes, static_cast<cudaStream_t>(stream)>>>(
        to_dev(layer), X, gy, rt, sv, g_o, g_z2, g_z1);
    return status();
}

int64_t pbr_gemm_tn_scratch(int64_t X, int32_t M, int32_t N) {
    const int64_t splits = X < 64 * kTile ? 1 : (X / (64 * kTile) < 64 ? X / (64 * kTile) : 64);
    return splits * static_cast<int64_t>(M) * N;
}

int pbr_gemm_tn_acc(const float* A, const float* B, int64_t X, int32_t M, int32_t N, float beta, float* C,
                    float* scratch, void* stream) {
    if (!A || !B || !C || !scratch || X < 1 || M < 1 || N < 1) return PBR_ERR_ARG;
    const int64_t splits = pbr_gemm_tn_scratch(X, M, N) / (static_cast<int64_t>(M) * N);
    const int64_t chunk = (X + splits - 1) / splits;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    dim3 grid((M + kTile - 1) / kTile, (N + kTile - 1) / kTile, static_cast<unsigned>(splits));
    gemm_tn_partial<<<grid, 256, 0, st>>>(A, B, X, M, N, chunk, scratch);
    gemm_tn_reduce<<<grid_for(static_cast<int64_t>(M) * N, 256), 256, 0, st>>>(scratch, static_cast<int>(splits),
                                                                               M * N, beta, C);
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
             float beta2, float eps, int32_t step, void* stream) {
    if (!param || !grad || !m || !v || n < 0 || step < 1) return PBR_ERR_ARG;
    if (n == 0) return PBR_OK;
    const float c1 = 1.f - powf(beta1, static_cast<float>(step));
    const float c2 = 1.f - powf(beta2, static_cast<float>(step));
    adam_kernel<<<grid_for(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(param, grad, m, v, n, lr,
                                                                                  beta1, beta2, eps, c1, c2);
    return status();
}

}  // extern "C"
