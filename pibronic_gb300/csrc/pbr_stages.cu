// pbr_stages.cu -- FP64 stage kernels: the reference's stage functions one at a time, in the
// reference's tensor layouts (pimc.py:1062-1213).  They serve the stage-level API of the Python
// package (build_o_matrix, build_denominator, diagonalize_coupling_matrix, build_numerator) and
// the stage-by-stage parity tests; the production path is the fused kernel.
#include <cmath>

#include "pbr_common.cuh"

namespace {

constexpr int kStageThreads = 128;
constexpr int kMaxAm = PBR_MAX_A_RHO;

inline int grid_for(int64_t n) { return static_cast<int>((n + kStageThreads - 1) / kStageThreads); }

// O[b,p,:,:] for one (b,p): dense Am x Am block, diagonal entries a < n_fill
// (pimc.py:1087-1129).  Exponent in the cancellation-free form
//   coth (x1^2 + x2^2) - 2 csch x1 x2 = csch (x1 - x2)^2 + (coth - csch)(x1^2 + x2^2).
__global__ void o_matrix_kernel(const double* __restrict__ q, int64_t B, int Am, int N, int P,
                                const double* __restrict__ coth, const double* __restrict__ csch,
                                const double* __restrict__ shift, const double* __restrict__ pref,
                                int n_fill, double* __restrict__ O) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= B * P) return;
    const int64_t b = idx / P;
    const int p = static_cast<int>(idx - b * P);
    const int pn = (p + 1 == P) ? 0 : p + 1;
    double* blk = O + idx * Am * Am;
    for (int i = 0; i < Am * Am; ++i) blk[i] = 0.0;
    for (int a = 0; a < n_fill; ++a) {
        const double* qa = q + (b * Am + a) * static_cast<int64_t>(N) * P;
        double s = 0.0;
        for (int j = 0; j < N; ++j) {
            const double x1 = qa[j * P + p] - shift[a * N + j];
            const double x2 = qa[j * P + pn] - shift[a * N + j];
            const double ch = coth[a * N + j], sh = csch[a * N + j];
            const double d = x1 - x2;
            s += sh * d * d + (ch - sh) * (x1 * x1 + x2 * x2);
        }
        blk[a * Am + a] = pref[a] * exp(-0.5 * s);
    }
}

__global__ void scale_kernel(double* O1, int A1, double* O2, int A2, int64_t BP, double* S12) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= BP) return;
    double* b1 = O1 + idx * A1 * A1;
    double* b2 = O2 + idx * A2 * A2;
    double mx = b1[0];
    for (int i = 0; i < A1 * A1; ++i) mx = fmax(mx, b1[i]);
    for (int i = 0; i < A2 * A2; ++i) mx = fmax(mx, b2[i]);
    for (int i = 0; i < A1 * A1; ++i) b1[i] /= mx;
    for (int i = 0; i < A2 * A2; ++i) b2[i] /= mx;
    S12[idx] = mx;
}

// per (sample, bead): each model's max O entry and the larger of the two (pimc.py:1076-1084)
__global__ void scaling_factors_kernel(const double* O1, int A1, const double* O2, int A2, int64_t BP,
                                       double* S1, double* S2, double* S12) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= BP) return;
    const double* b1 = O1 + idx * A1 * A1;
    const double* b2 = O2 + idx * A2 * A2;
    double m1 = b1[0], m2 = b2[0];
    for (int i = 1; i < A1 * A1; ++i) m1 = fmax(m1, b1[i]);
    for (int i = 1; i < A2 * A2; ++i) m2 = fmax(m2, b2[i]);
    if (S1) S1[idx] = m1;
    if (S2) S2[idx] = m2;
    S12[idx] = fmax(m1, m2);
}

__global__ void divide_kernel(double* O, int A, int64_t BP, const double* S12) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= BP) return;
    double* b = O + idx * A * A;
    const double s = S12[idx];
    for (int i = 0; i < A * A; ++i) b[i] /= s;
}

// rho[b] = Tr prod_p O[b,p] for diagonal O (pimc.py:1132-1136)
__global__ void denominator_kernel(const double* O, int64_t B, int A, int P, double* out) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double tr = 0.0;
    for (int a = 0; a < A; ++a) {
        double pr = 1.0;
        for (int p = 0; p < P; ++p) pr *= O[((b * P + p) * A + a) * A + a];
        tr += pr;
    }
    out[b] = tr;
}

// V and its eigen-decomposition for one (b,p) (pimc.py:1139-1174):
//   V[x,y] = sum_{d,e} q[b,y,e,p] 1/2 Q[d,e,x,y] q[b,x,d,p] + sum_d L[d,x,y] q[b,x,d,p] + E[x,y]
template <int A>
__global__ void coupling_eigh_kernel(const double* __restrict__ q, int64_t B, int N, int P,
                                     const double* __restrict__ E, const double* __restrict__ L,
                                     const double* __restrict__ Q, double* __restrict__ V,
                                     double* __restrict__ evals, double* __restrict__ evecs,
                                     int32_t* sym_ok) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= B * P) return;
    const int64_t b = idx / P;
    const int p = static_cast<int>(idx - b * P);
    double a[A][A];
    bool sym = true;
#pragma unroll
    for (int x = 0; x < A; ++x)
#pragma unroll
        for (int y = 0; y < A; ++y) {
            const double* qx = q + (b * A + x) * static_cast<int64_t>(N) * P;
            const double* qy = q + (b * A + y) * static_cast<int64_t>(N) * P;
            double v = E[x * A + y];
            for (int d = 0; d < N; ++d) {
                const double qd = qx[d * P + p];
                double inner = L[(d * A + x) * A + y];
                for (int e = 0; e < N; ++e)
                    inner += 0.5 * Q[((static_cast<int64_t>(d) * N + e) * A + x) * A + y] * qy[e * P + p];
                v += inner * qd;
            }
            a[x][y] = v;
        }
    double* vout = V + idx * A * A;
#pragma unroll
    for (int x = 0; x < A; ++x)
#pragma unroll
        for (int y = 0; y < A; ++y) {
            vout[x * A + y] = a[x][y];
            if (fabs(a[x][y] - a[y][x]) > 1e-8 + 1e-5 * fabs(a[y][x])) sym = false;   // np.allclose
        }
    if (!sym) atomicAnd(sym_ok, 0);
    // LAPACK eigh(UPLO='L') reads the lower triangle
#pragma unroll
    for (int x = 0; x < A; ++x)
#pragma unroll
        for (int y = x + 1; y < A; ++y) a[x][y] = a[y][x];
    double u[A][A];
    pbr::jacobi_eigh<double, A>(a, u, 30);
    // ascending order, eigenvectors as columns
    int order[A];
#pragma unroll
    for (int i = 0; i < A; ++i) order[i] = i;
#pragma unroll
    for (int i = 0; i < A; ++i)
#pragma unroll
        for (int j = 0; j < A - 1 - i; ++j)
            if (a[order[j]][order[j]] > a[order[j + 1]][order[j + 1]]) {
                const int t = order[j]; order[j] = order[j + 1]; order[j + 1] = t;
            }
#pragma unroll
    for (int i = 0; i < A; ++i) {
        int oi = 0;
#pragma unroll
        for (int k = 0; k < A; ++k) if (order[i] == k) oi = k;
        double lam = 0.0;
#pragma unroll
        for (int k = 0; k < A; ++k) if (k == oi) lam = a[k][k];
        evals[idx * A + i] = lam;
#pragma unroll
        for (int r = 0; r < A; ++r) {
            double ur = 0.0;
#pragma unroll
            for (int k = 0; k < A; ++k) if (k == oi) ur = u[r][k];
            evecs[(idx * A + r) * A + i] = ur;
        }
    }
}

// M = U diag(exp(-tau lambda)) U^T; g[b] = Tr prod_p (M_p O_p) (pimc.py:1177-1213)
template <int A>
__global__ void numerator_kernel(const double* __restrict__ evals, const double* __restrict__ evecs,
                                 const double* __restrict__ O, int64_t B, int P, double tau,
                                 double* __restrict__ Mout, double* __restrict__ out) {
    const int64_t b = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double acc[A][A];
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c < A; ++c) acc[r][c] = (r == c) ? 1.0 : 0.0;
    for (int p = 0; p < P; ++p) {
        const int64_t bp = b * P + p;
        double ev[A], M[A][A];
#pragma unroll
        for (int i = 0; i < A; ++i) ev[i] = exp(-tau * evals[bp * A + i]);
#pragma unroll
        for (int r = 0; r < A; ++r)
#pragma unroll
            for (int c = 0; c < A; ++c) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < A; ++i) s += evecs[(bp * A + r) * A + i] * ev[i] * evecs[(bp * A + c) * A + i];
                M[r][c] = s;
                if (Mout) Mout[(bp * A + r) * A + c] = s;
            }
        double t[A][A];
#pragma unroll
        for (int r = 0; r < A; ++r)
#pragma unroll
            for (int c = 0; c < A; ++c) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < A; ++k) s += acc[r][k] * M[k][c];
                t[r][c] = s;
            }
        const double* Op = O + bp * A * A;
#pragma unroll
        for (int r = 0; r < A; ++r)
#pragma unroll
            for (int c = 0; c < A; ++c) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < A; ++k) s += t[r][k] * Op[k * A + c];
                acc[r][c] = s;
            }
    }
    double tr = 0.0;
#pragma unroll
    for (int r = 0; r < A; ++r) tr += acc[r][r];
    out[b] = tr;
}

#define PBR_DISPATCH_A(A, EXPR_T)              \
    switch (A) {                               \
        case 1: { constexpr int kA = 1; EXPR_T; } break; \
        case 2: { constexpr int kA = 2; EXPR_T; } break; \
        case 3: { constexpr int kA = 3; EXPR_T; } break; \
        case 4: { constexpr int kA = 4; EXPR_T; } break; \
        case 5: { constexpr int kA = 5; EXPR_T; } break; \
        case 6: { constexpr int kA = 6; EXPR_T; } break; \
        case 7: { constexpr int kA = 7; EXPR_T; } break; \
        case 8: { constexpr int kA = 8; EXPR_T; } break; \
        default: return PBR_ERR_UNSUPPORTED;   \
    }

inline int last_status() { return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA; }

}  // namespace

extern "C" {

int pbr_o_matrix(const double* q_slots, int64_t B, int32_t Am, int32_t N, int32_t P,
                 const double* coth, const double* csch, const double* shift,
                 const double* prefactor, int32_t n_fill, double* O, void* stream) {
    if (!q_slots || !coth || !csch || !shift || !prefactor || !O) return PBR_ERR_ARG;
    if (B < 0 || Am < 1 || Am > kMaxAm || N < 1 || P < 3 || n_fill < 0 || n_fill > Am) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    o_matrix_kernel<<<grid_for(B * P), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        q_slots, B, Am, N, P, coth, csch, shift, prefactor, n_fill, O);
    return last_status();
}

int pbr_scale_o_matrices(double* O1, int32_t A1, double* O2, int32_t A2, int64_t B, int32_t P,
                         double* S12, void* stream) {
    if (!O1 || !O2 || !S12 || A1 < 1 || A2 < 1 || B < 0 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    scale_kernel<<<grid_for(B * P), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        O1, A1, O2, A2, B * P, S12);
    return last_status();
}

int pbr_scaling_factors(const double* O1, int32_t A1, const double* O2, int32_t A2, int64_t B, int32_t P,
                        double* S1, double* S2, double* S12, void* stream) {
    if (!O1 || !O2 || !S12 || A1 < 1 || A2 < 1 || B < 0 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    scaling_factors_kernel<<<grid_for(B * P), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        O1, A1, O2, A2, B * P, S1, S2, S12);
    return last_status();
}

int pbr_divide_o_matrix(double* O, int32_t A, int64_t B, int32_t P, const double* S12,
                        void* stream) {
    if (!O || !S12 || A < 1 || B < 0 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    divide_kernel<<<grid_for(B * P), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        O, A, B * P, S12);
    return last_status();
}

int pbr_denominator(const double* O, int64_t B, int32_t A, int32_t P, double* out, void* stream) {
    if (!O || !out || A < 1 || B < 0 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    denominator_kernel<<<grid_for(B), kStageThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        O, B, A, P, out);
    return last_status();
}

int pbr_coupling_eigh(const double* q_slots, int64_t B, int32_t A, int32_t N, int32_t P,
                      const double* E, const double* L, const double* Q, double* V,
                      double* eigvals, double* eigvecs, int32_t* sym_ok, void* stream) {
    if (!q_slots || !E || !L || !Q || !V || !eigvals || !eigvecs || !sym_ok) return PBR_ERR_ARG;
    if (B < 0 || N < 1 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PBR_DISPATCH_A(A, (coupling_eigh_kernel<kA><<<grid_for(B * P), kStageThreads, 0, st>>>(
                          q_slots, B, N, P, E, L, Q, V, eigvals, eigvecs, sym_ok)));
    return last_status();
}

int pbr_numerator(const double* eigvals, const double* eigvecs, const double* O, int64_t B,
                  int32_t A, int32_t P, double tau, double* M, double* out, void* stream) {
    if (!eigvals || !eigvecs || !O || !out || B < 0 || P < 1) return PBR_ERR_ARG;
    if (B == 0) return PBR_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PBR_DISPATCH_A(A, (numerator_kernel<kA><<<grid_for(B), kStageThreads, 0, st>>>(
                          eigvals, eigvecs, O, B, P, tau, M, out)));
    return last_status();
}

}  // extern "C"
