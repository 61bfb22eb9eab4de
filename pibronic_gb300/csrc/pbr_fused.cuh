// pbr_fused.cuh -- the fused PIMC block-evaluation kernel.
//
// One CTA of kThreads threads handles S = kThreads / G samples at a time; the G threads of a
// sample (G a power of two, a segment of one warp) each own a contiguous chunk of C beads.
//
//   phase A  bead coordinates q[j][p] of every sample into shared memory: either drawn on the
//            device (Philox normals scaled by the normal-mode standard deviations of the sampled
//            source surface, then the real-Fourier ring transform, then the source shift;
//            pimc.py:326-334, 613-631) or read from the caller's q.
//   phase B  per bead p of the thread's chunk (pimc.py:1087-1213):
//              phi^rho_pa, phi^vib_pa(beta + h) as a Taylor series in h (order K), in the
//              cancellation-free form of the O-matrix exponent;
//              ln S12_p = max over both models (pimc.py:1076-1084);
//              O-hat_pa(h) = exp(phi^vib_pa(h) - ln S12_p) as a series;
//              V(q_p) (energies, linear, packed quadratic), Jacobi eigensolver,
//              M_p = U exp(-tau lambda) U^T with a power-of-two shift;
//              chunk product  N(h) <- N(h) M_p diag(O-hat_p(h)), renormalised by a power of two.
//   phase C  chunk products combined in bead order by a shuffle tree within the segment.
//   phase D  traces: s_g = Tr N_0, g(beta +- db) = sum_k Tr N_k (+-db)^k, s_rho = sum_a exp(sum_p
//            (phi^rho_pa - ln S12_p)); the traces summed in the kernel's type, scaled exactly by
//            the accumulated power-of-two exponent and combined in FP64.
#pragma once

#include "pbr_common.cuh"

namespace pbr {

constexpr int kThreads = 128;
// the tensor-core quadratic is used at 3-4 surfaces from this many modes on (measured: 8 % faster
// at A = 4, N = 20; 1-6 % slower at N = 8-12, where the FP32 pair loop is short);
// records whose |q| exceeds kTcqMaxQ keep every q_d q_e below 2^15, inside FP16's range -- a warp
// holding a larger one takes the FP32 pair loop for that bead
constexpr int kTcqMinN = 16;
constexpr float kTcqMaxQ = 181.0f;
// target beads per thread (chunk length) of the ring product: 16 rather than 8 halves the
// threads per sample, so fewer chunk products to combine, fewer chains idle in the sampler's
// second pass and the per-sample outputs spread over more beads (A = 4, N = 12, P = 64: 15.25 ->
// 13.4 ms per 1e6 samples)
constexpr int kMaxChunk = 16;
// kQ32V: q from the caller (FP32) and V(q) precomputed per (sample, bead) row by the
// tensor-core contraction (row-team form only)
enum QMode : int { kSample = 0, kQ64 = 1, kQ32 = 2, kQ32V = 3 };

struct FusedArgs {
    pbr_model m;
    const void* q_in;
    int64_t X;
    pbr_outputs out;
    uint32_t key0, key1;
    uint64_t offset;
    int G, logG, C, S;
    int rs;         // row stride of one mode's beads in shared memory (skewed, see qidx)
    int qstride;    // elements per sample in the q region
    int tcq;        // 1: the tensor-core quadratic (its tables, its kernel instantiation)
};

__host__ __device__ inline int align_up(int x, int a) { return (x + a - 1) / a * a; }

// Bead p of mode j in a sample's shared-memory block.  Beads are skewed by one slot every 32 so
// that threads owning chunks 32 beads apart do not hit the same bank.
__host__ __device__ __forceinline__ int qidx(int j, int p, int rs) { return j * rs + p + (p >> 5); }
__host__ __device__ inline int row_stride(int P) { return P + ((P + 31) >> 5); }

// Per-mode record of the tables read in the bead loop (one 128-bit-aligned block per mode):
//   [0,KP) vib csch series/2 | [KP,2KP) vib tanh series/2 | [2KP,2KP+AP) vib d_a |
//   [2KP+AP,2KP+2AP) rho d_a | 4: rho csch/2, rho tanh/2, 0, 0 | A2P: linear couplings (pairs)
__host__ __device__ inline int rec_len(int A, int K) {
    return 2 * align_up(K + 1, 4) + 2 * align_up(A, 4) + 4 + align_up(npair(A), 4);
}

// Shared-memory plan (in elements of the table type, esz bytes each); identical on host and device.
// Tensor-core quadratic part of V in the register-chunk form (FP32 build, A <= 4): the mode
// pairs (d, e <= d) are grouped in quadruples (d, e0 .. e0+3) -- one FP16 MMA k-step of 16 pair
// slots holds four quadruples -- and the warp's 32 (sample, bead) records form the MMA's rows.
__host__ __device__ inline int tcq_quads(int N) {
    int n = 0;
    for (int d = 0; d < N; ++d) n += (d + 4) / 4;        // ceil((d + 1) / 4) per row d
    return n;
}
__host__ __device__ inline int tcq_ksteps(int N) { return (tcq_quads(N) + 3) / 4; }
__host__ __device__ constexpr int tcq_ntiles(int A) { return (npair(A) + 7) / 8; }
// 32-bit words: B fragments (k-steps x n-tiles x 32 lanes x 4), quadruple descriptors (int4 per
// quadruple), the inverse coupling scale
__host__ __device__ inline int tcq_words(int N, int A) {
    return tcq_ksteps(N) * tcq_ntiles(A) * 128 + tcq_ksteps(N) * 16 + 4;
}

struct SmemPlan {
    int c, e, qq, rc, rec, q, qlo, total_bytes;
    int tcq_k;   // k-steps of the tensor-core quadratic (0: the FP32 pair loop over a packed table)
    __host__ __device__ SmemPlan(int A, int K, int qm, int esz, int N, int P, int S, int qstride, int tcq) {
        const int A2P = align_up(npair(A), 4);
        int o = 0;
        auto take = [&](int n) { int r = o; o = align_up(o + n, 4); return r; };
        // the quadruple descriptors hold mode offsets d * rs in 16 bits
        tcq_k = (tcq && esz == 4 && A >= 3 && A <= 4 && N >= kTcqMinN && qstride - 1 < 65536) ? tcq_ksteps(N) : 0;
        c = take((K + 1) * A); e = take(A2P); qq = take(tcq_k ? tcq_words(N, A) : npair(N) * A2P); rc = take(A);
        rec = take(N * rec_len(A, K));
        q = take(S * qstride);
        qlo = take((qm == kQ64 && esz == 4) ? S * qstride : 0);
        total_bytes = o * esz;
    }
};

template <typename T> __device__ __forceinline__ T dev_fabs(T x) { return x < T(0) ? -x : x; }

// CNT consecutive values to shared memory, 128-bit stores for FP32 when CNT % 4 == 0.
template <typename T, int CNT>
__device__ __forceinline__ void stv(T* __restrict__ dst, const T (&src)[CNT]) {
    if constexpr (sizeof(T) == 4 && CNT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < CNT; i += 4)
            *reinterpret_cast<float4*>(dst + i) = make_float4(src[i], src[i + 1], src[i + 2], src[i + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < CNT; ++i) dst[i] = src[i];
    }
}

// CNT consecutive table values from shared memory, 128-bit loads where the type allows.
template <typename T, int CNT>
__device__ __forceinline__ void ldv(const T* __restrict__ src, T (&dst)[CNT]) {
    if constexpr (sizeof(T) == 4 && CNT % 4 == 0) {
#pragma unroll
        for (int i = 0; i < CNT; i += 4) {
            const float4 v = *reinterpret_cast<const float4*>(src + i);
            dst[i] = v.x; dst[i + 1] = v.y; dst[i + 2] = v.z; dst[i + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 8 && CNT % 2 == 0) {
#pragma unroll
        for (int i = 0; i < CNT; i += 2) {
            const double2 v = *reinterpret_cast<const double2*>(src + i);
            dst[i] = v.x; dst[i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < CNT; ++i) dst[i] = src[i];
    }
}

// Jacobi rotation (c, s, t) annihilating a_pq of the 2x2 block [[app, apq], [apq, aqq]].
// FP32 uses the fast reciprocal and rsqrt: any (c, s) with c^2 + s^2 = 1 keeps the sweep
// orthogonal, an inexact angle only leaves a small a_pq for the next sweep.
__device__ __forceinline__ void jrot(float app, float aqq, float apq, float& c, float& s, float& t) {
    const float zeta = __fdividef(aqq - app, 2.0f * apq);
    const float az = fabsf(zeta);
    float tt;
    if (az > 1e18f) {
        tt = __fdividef(0.5f, zeta);
    } else {
        const float x = fmaf(zeta, zeta, 1.0f);
        tt = copysignf(__fdividef(1.0f, az + x * rsqrtf(x)), zeta);
    }
    c = rsqrtf(fmaf(tt, tt, 1.0f));
    s = tt * c;
    t = tt;
}
__device__ __forceinline__ void jrot(double app, double aqq, double apq, double& c, double& s, double& t) {
    const double zeta = (aqq - app) / (2.0 * apq);
    const double az = fabs(zeta);
    double tt;
    if (az > 1e150) {
        tt = 0.5 / zeta;
    } else {
        tt = 1.0 / (az + sqrt(1.0 + zeta * zeta));
        if (zeta < 0.0) tt = -tt;
    }
    c = 1.0 / sqrt(1.0 + tt * tt);
    s = tt * c;
    t = tt;
}

// Cyclic Jacobi on symmetric a (registers) accumulating the rotations into u, which holds the
// starting basis on entry (identity, or the previous bead's eigenvectors: a warm start).
template <typename T, int A>
__device__ __forceinline__ void jacobi_accumulate(T (&a)[A][A], T (&u)[A][A], int max_sweeps) {
    if (A == 1) return;
    const T tol = eps_of<T>::value * eps_of<T>::value;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        T off = T(0), dia = T(0);
#pragma unroll
        for (int p = 0; p < A; ++p) {
            dia = fma(a[p][p], a[p][p], dia);
#pragma unroll
            for (int q = p + 1; q < A; ++q) off = fma(a[p][q], a[p][q], off);
        }
        if (off <= tol * dia || off == T(0)) break;
#pragma unroll
        for (int p = 0; p < A - 1; ++p) {
#pragma unroll
            for (int q = p + 1; q < A; ++q) {
                const T apq = a[p][q];
                if (apq == T(0)) continue;
                T c, s, t;
                jrot(a[p][p], a[q][q], apq, c, s, t);
                a[p][p] = fma(-t, apq, a[p][p]);
                a[q][q] = fma(t, apq, a[q][q]);
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

// Forms chosen at compile time from measurements: the register exponential below replaces the
// Jacobi eigensolver from 3 surfaces on (a 2 x 2 Jacobi is a single exact rotation), and the
// quadratic part of V runs as one flat loop over the mode pairs from 4 surfaces on (below that the
// pair-index bookkeeping outweighs the few FMAs per pair).
constexpr int kExpmMinA = 3;
constexpr int kFlatPairsMinA = 4;

// index of entry (r, c) of a symmetric A x A matrix stored as its lower triangle (pair order)
__host__ __device__ constexpr int sym_index(int r, int c) { return r >= c ? r * (r + 1) / 2 + c : c * (c + 1) / 2 + r; }

// Z = X Y for symmetric X, Y that are polynomials in one matrix (so Z is symmetric): the lower
// triangle only, each entry summed over m in order
template <int A>
__device__ __forceinline__ void sym_mul(const float (&X)[npair(A)], const float (&Y)[npair(A)], float (&Z)[npair(A)]) {
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int m = 0; m < A; ++m) acc = fmaf(X[sym_index(r, m)], Y[sym_index(m, c)], acc);
            Z[sym_index(r, c)] = acc;
        }
}

// exp(-tau V) for a small symmetric V given as its lower triangle vp (pair order), in FP32
// registers: V is shifted by its mean eigenvalue (trace / A), scaled by 2^-s until
// ||tau (V - mean)||_inf <= 1/2, exponentiated by the degree-8 Taylor polynomial
// (Paterson-Stockmeyer: C_0 + B^3 (C_1 + B^3 C_2), truncation < 1e-8) and squared s times.  Every
// intermediate is a polynomial in B, hence symmetric, and is kept as its lower triangle (A(A+1)/2
// registers and A^2 (A+1)/2 FMAs per product).  M = 2^(tl - n2) X with tl = -tau mean log2(e);
// returns n2, the power of two taken out.  For symmetric V this is the matrix the reference forms
// from eigh (pimc.py:1197-1205).
// The lower triangle X of the scaled exponential and its factor: M = f X, f = 2^(tl - n2).
template <int A>
__device__ __forceinline__ int expm_neg_tau_packed(const float (&vp)[npair(A)], float tau, float (&X)[npair(A)],
                                                   float& f) {
    constexpr int NS = npair(A);
    float mean = 0.f;
#pragma unroll
    for (int i = 0; i < A; ++i) mean += vp[sym_index(i, i)];
    mean *= 1.f / float(A);
    float B[NS];
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) B[sym_index(r, c)] = -tau * (vp[sym_index(r, c)] - (r == c ? mean : 0.f));
    float nrm = 0.f;
#pragma unroll
    for (int r = 0; r < A; ++r) {
        float rs = 0.f;
#pragma unroll
        for (int c = 0; c < A; ++c) rs += fabsf(B[sym_index(r, c)]);
        nrm = fmaxf(nrm, rs);
    }
    int s = 0;
    while (nrm > 0.5f && s < 40) { nrm *= 0.5f; ++s; }
    const float sc = ldexpf(1.f, -s);
#pragma unroll
    for (int i = 0; i < NS; ++i) B[i] *= sc;
    float B2[NS], B3[NS], T1[NS];
    sym_mul<A>(B, B, B2);
    sym_mul<A>(B2, B, B3);
    constexpr float c3 = 1.f / 6.f, c4 = 1.f / 24.f, c5 = 1.f / 120.f, c6 = 1.f / 720.f, c7 = 1.f / 5040.f,
                    c8 = 1.f / 40320.f;
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            const int i = sym_index(r, c);
            T1[i] = (r == c ? c6 : 0.f) + c7 * B[i] + c8 * B2[i];
        }
    sym_mul<A>(T1, B3, X);
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            const int i = sym_index(r, c);
            T1[i] = X[i] + (r == c ? c3 : 0.f) + c4 * B[i] + c5 * B2[i];
        }
    sym_mul<A>(T1, B3, X);
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            const int i = sym_index(r, c);
            X[i] += (r == c ? 1.f : 0.f) + B[i] + 0.5f * B2[i];
        }
    for (int i = 0; i < s; ++i) {
        sym_mul<A>(X, X, T1);
#pragma unroll
        for (int j = 0; j < NS; ++j) X[j] = T1[j];
    }
    const float tl = -tau * mean * 1.4426950408889634f;
    const float n2 = floorf(tl);
    f = exp2f(tl - n2);
    return static_cast<int>(n2);
}

template <int A>
__device__ __forceinline__ int expm_neg_tau(const float (&vp)[npair(A)], float tau, float (&M)[A][A]) {
    float X[npair(A)], f;
    const int n2 = expm_neg_tau_packed<A>(vp, tau, X, f);
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c < A; ++c) M[r][c] = f * X[sym_index(r, c)];
    return n2;
}

// Compensated (Kahan) FP32 sum for the per-chunk log accumulators; plain sum in FP64.
template <typename T> struct LogSum;
template <> struct LogSum<float> {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return static_cast<double>(s) - static_cast<double>(c); }
    // adds another compensated sum: the leading parts by an error-free two-sum, whose rounding
    // error goes into the compensation (the chunk combine stays in FP32)
    __device__ __forceinline__ void merge(const LogSum& o) {
        const float t = s + o.s;
        const float bp = t - s;
        const float e = (s - (t - bp)) + (o.s - bp);
        c = (c + o.c) - e;
        s = t;
    }
    __device__ __forceinline__ LogSum shfl_down(int st, int width) const {
        LogSum r;
        r.s = __shfl_down_sync(0xffffffffu, s, st, width);
        r.c = __shfl_down_sync(0xffffffffu, c, st, width);
        return r;
    }
};
template <> struct LogSum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double value() const { return s; }
    __device__ __forceinline__ void merge(const LogSum& o) { s += o.s; }
    __device__ __forceinline__ LogSum shfl_down(int st, int width) const {
        LogSum r;
        r.s = __shfl_down_sync(0xffffffffu, s, st, width);
        return r;
    }
};

// Source surface of global sample sg ~ Categorical(state weights) (pimc.py:386-389).
template <typename T>
__device__ __forceinline__ int draw_source(const pbr_model& m, uint64_t sg, uint32_t key0, uint32_t key1) {
    const u32x4 r = philox4x32_10(u32x4{0xFFFFFFFFu, static_cast<uint32_t>(sg),
                                        static_cast<uint32_t>(sg >> 32), 1u}, key0, key1);
    const float u = u01(r.x);
    const T* cdf = static_cast<const T*>(m.src_cdf);
    int src = 0;
    for (int a = 0; a < m.A_rho - 1; ++a) src += (u >= static_cast<float>(cdf[a])) ? 1 : 0;
    return src;
}

// Bead coordinates of mode j of global sample sg (pimc.py:326-334, 613-631): standard normals
// z_p (Philox counter (j * ceil(P/4) + p/4, sample), Box-Muller) and back substitution
// x = L^-T z through the cyclic-tridiagonal factor of rho's bead precision,
//   x_p = a_p (z_p - b_p x_{p+1} - c_p x_{P-1}),  q_p = x_p + d_src,j,
// handed to sink(p, q_p) for p = P-1 down to 0.  The FMAs are explicit so every kernel form
// that draws through this function produces the same bits.  The distribution is rho's
// N(d_src, Lambda^-1), the one the reference draws in normal modes.
// one step of the back substitution: x_{P-1} = a z, else x_p = a_p (z_p - b_p x_{p+1} - c_p x_{P-1});
// xnext <- x_p (and xlast <- x_p at p = P-1).  The product by a_p is rounded on its own (no
// contraction into the q_p = x_p + d add that follows), so every caller gets the same bits.
__device__ __forceinline__ float mul_rn(float x, float y) { return __fmul_rn(x, y); }
__device__ __forceinline__ double mul_rn(double x, double y) { return __dmul_rn(x, y); }

template <typename T>
__device__ __forceinline__ void chain_next(T av, T bv, T cv, T z, T& xnext, T xlast) {
    xnext = mul_rn(av, fma(-cv, xlast, fma(-bv, xnext, z)));
}

// a, b, c point at mode j's first coefficient (global or shared memory); bead p's is p * ld
// further (ld = N: the table is bead-major, so the threads of a tile that run different modes read
// neighbouring words)
template <typename T>
__device__ __forceinline__ void chain_step(const T* __restrict__ a, const T* __restrict__ b,
                                           const T* __restrict__ c, int p, int P, int ld, T z, T& xnext,
                                           T& xlast) {
    const int o = p * ld;
    if (p == P - 1) {
        xnext = mul_rn(a[o], z);
        xlast = xnext;
    } else {
        chain_next<T>(a[o], b[o], c[o], z, xnext, xlast);
    }
}

template <typename T, typename Sink>
__device__ __forceinline__ void draw_mode_chain_to(const pbr_model& m, int j, uint64_t sg, uint32_t key0,
                                                   uint32_t key1, T dsh, Sink&& sink) {
    const int N = m.N, P = m.P;
    const T* a = static_cast<const T*>(m.ring_chol) + j;
    const T* b = a + static_cast<int64_t>(N) * P;
    const T* c = b + static_cast<int64_t>(N) * P;
    const uint32_t lo = static_cast<uint32_t>(sg), hi = static_cast<uint32_t>(sg >> 32);
    const int CP = (P + 3) >> 2;
    T xnext = T(0), xlast = T(0);
    for (int p4 = (P - 1) >> 2; p4 >= 0; --p4) {
        // the group's coefficients are loaded first, so their latency hides behind Philox
        T ka[4], kb[4], kc[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int p = 4 * p4 + t;
            const int o = (p < P ? p : 0) * N;
            ka[t] = a[o]; kb[t] = b[o]; kc[t] = c[o];
        }
        const u32x4 r = philox4x32_10(u32x4{static_cast<uint32_t>(j * CP + p4), lo, hi, 0u}, key0, key1);
        float z[4];
        box_muller(r.x, r.y, z[0], z[1]);
        box_muller(r.z, r.w, z[2], z[3]);
#pragma unroll
        for (int t = 3; t >= 0; --t) {
            const int p = 4 * p4 + t;
            if (p >= P) continue;
            if (p == P - 1) {
                xnext = mul_rn(ka[t], T(z[t]));
                xlast = xnext;
            } else {
                chain_next<T>(ka[t], kb[t], kc[t], T(z[t]), xnext, xlast);
            }
            sink(p, xnext + dsh);
        }
    }
}


// The sampler in two passes, for kernel forms whose threads share a tile of samples: first the
// standard normals of every (sample, mode, group of 4 beads) counter -- the Philox / Box-Muller
// work, spread evenly over the threads -- are written to the samples' mode-major buffers, then
// each (sample, mode) chain is back-substituted in place.  The counters and the chain steps are
// those of draw_mode_chain_to, so the bits are the same.
//
// normals of samples s < ns (global index sg0 + s) into qs + s * qstride, work items
// u = u0, u0 + du, ... of the ns N ceil(P/4) counters
template <typename T, bool kOneSample = false>
__device__ __forceinline__ void fill_normals(const pbr_model& m, T* qs, int qstride, int rs, int ns, uint64_t sg0,
                                             uint32_t key0, uint32_t key1, int u0, int du) {
    const int N = m.N, P = m.P, CP = (P + 3) >> 2, per = N * CP;
    for (int u = u0; u < ns * per; u += du) {
        const int s = kOneSample ? 0 : u / per, rem = u - s * per;
        const int j = rem / CP, p4 = rem - j * CP;
        const uint64_t sg = sg0 + static_cast<uint64_t>(s);
        const u32x4 r = philox4x32_10(u32x4{static_cast<uint32_t>(rem), static_cast<uint32_t>(sg),
                                            static_cast<uint32_t>(sg >> 32), 0u}, key0, key1);
        float z[4];
        box_muller(r.x, r.y, z[0], z[1]);
        box_muller(r.z, r.w, z[2], z[3]);
        T* qsj = qs + static_cast<int64_t>(s) * qstride;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int p = 4 * p4 + t;
            if (p < P) qsj[qidx(j, p, rs)] = T(z[t]);
        }
    }
}

// mode j of one sample, in place: normals in, q = x + dsh out (qj = the mode's row, skewed layout;
// tab = the ring factor [3][P][N], in global or shared memory).  The chain is serial, so the
// coefficients and normals of the next kBsGroup steps are loaded while the current group runs;
// the arithmetic is chain_step's.
constexpr int kBsGroup = 4;
template <typename T, int W = kBsGroup>
__device__ __forceinline__ void back_substitute(const T* tab, int N, int P, int j, T dsh, T* qj) {
    const T* a = tab + j;
    const T* b = a + static_cast<int64_t>(N) * P;
    const T* c = b + static_cast<int64_t>(N) * P;
    T xnext = T(0), xlast = T(0);
    {
        T* slot = qj + (P - 1) + ((P - 1) >> 5);
        chain_step<T>(a, b, c, P - 1, P, N, *slot, xnext, xlast);
        *slot = xnext + dsh;
    }
    int p = P - 2;
    if (p >= W - 1) {
        T ca[W], cb[W], cc[W], cz[W];
#pragma unroll
        for (int t = 0; t < W; ++t) {
            const int q = p - t;
            ca[t] = a[q * N]; cb[t] = b[q * N]; cc[t] = c[q * N]; cz[t] = qj[q + (q >> 5)];
        }
        while (true) {
            const int pn = p - W;
            const bool more = pn >= W - 1;
            T na[W], nb[W], nc[W], nz[W];
            if (more) {
#pragma unroll
                for (int t = 0; t < W; ++t) {
                    const int q = pn - t;
                    na[t] = a[q * N]; nb[t] = b[q * N]; nc[t] = c[q * N]; nz[t] = qj[q + (q >> 5)];
                }
            }
#pragma unroll
            for (int t = 0; t < W; ++t) {
                const int q = p - t;
                chain_next<T>(ca[t], cb[t], cc[t], cz[t], xnext, xlast);
                qj[q + (q >> 5)] = xnext + dsh;
            }
            p = pn;
            if (!more) break;
#pragma unroll
            for (int t = 0; t < W; ++t) { ca[t] = na[t]; cb[t] = nb[t]; cc[t] = nc[t]; cz[t] = nz[t]; }
        }
    }
    for (; p >= 0; --p) {
        T* slot = qj + p + (p >> 5);
        chain_step<T>(a, b, c, p, P, N, *slot, xnext, xlast);
        *slot = xnext + dsh;
    }
}

// Phase A of the chunk form, by the G threads of one sample (lanes gmask); returns the source
// surface.
template <typename T>
__device__ int draw_sample_smem(const pbr_model& m, T* qs, int rs, int64_t sidx, uint64_t offset,
                                uint32_t key0, uint32_t key1, int g, int G, unsigned gmask) {
    const uint64_t sg = offset + static_cast<uint64_t>(sidx);
    const int N = m.N;
    fill_normals<T, true>(m, qs, 0, rs, 1, sg, key0, key1, g, G);
    const int src = draw_source<T>(m, sg, key0, key1);
    const T* dsrc = static_cast<const T*>(m.rho_d) + static_cast<int64_t>(src) * N;
    __syncwarp(gmask);
    for (int j = g; j < N; j += G)
        back_substitute<T>(static_cast<const T*>(m.ring_chol), N, m.P, j, dsrc[j], qs + j * rs);
    __syncwarp(gmask);
    return src;
}

// power-of-two renormalisation of a series matrix; returns the exponent taken out
template <typename T, int K, int A>
__device__ __forceinline__ int renormalise(T (&n)[K + 1][A][A]) {
    T mx = T(0);
#pragma unroll
    for (int r = 0; r < A; ++r)
#pragma unroll
        for (int c = 0; c < A; ++c) mx = max(mx, dev_fabs(n[0][r][c]));
    if (!(mx > T(0)) || !isfinite(mx)) return 0;
    int e2;
    frexp(mx, &e2);
    const T sc = ldexp(T(1), -e2);
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
        for (int r = 0; r < A; ++r)
#pragma unroll
            for (int c = 0; c < A; ++c) n[k][r][c] *= sc;
    return e2;
}

// Shared-memory tables of the tensor-core quadratic, built by the whole block (ends with a
// barrier): the couplings Q[pair][bc] scaled by 2^s (max |Q| 2^s in [2^13, 2^14), so their FP16
// low parts stay normal), split into FP16 hi and lo and laid out as each lane's B fragment of
// mma.m16n8k16 (rows 2t, 2t+1 = slots 0, 1 and rows 2t+8, 2t+9 = slots 2, 3 of quadruple 4 kk + t,
// column g = surface pair 8 nt + g); per quadruple the offsets d rs and min(e0 + s, d) rs of its
// four slots; then 2^-s.
template <int A>
__device__ void tcq_tables(const float* __restrict__ g_qq, int N, int rs, int nks, uint32_t* tq) {
    constexpr int A2 = npair(A);
    constexpr int NT = tcq_ntiles(A);
    const int nq4 = 4 * nks;
    int4* desc = reinterpret_cast<int4*>(tq + nks * NT * 128);
    float* sinv = reinterpret_cast<float*>(desc + nq4);
    if (threadIdx.x == 0) *reinterpret_cast<int*>(sinv) = 0;
    __syncthreads();
    float mx = 0.f;
    for (int i = threadIdx.x; i < npair(N) * A2; i += blockDim.x) mx = fmaxf(mx, fabsf(g_qq[i]));
    atomicMax(reinterpret_cast<int*>(sinv), __float_as_int(mx));       // non-negative floats order as ints
    for (int u = threadIdx.x; u < nq4; u += blockDim.x) {
        int4 r = make_int4(0, 0, 0, -1);                                  // padding: zero couplings
        int base = 0;
        for (int d = 0; d < N; ++d) {
            const int nq = (d + 4) / 4;
            if (u < base + nq) {
                const int e0 = 4 * (u - base);
                int o[4];
#pragma unroll
                for (int s = 0; s < 4; ++s) o[s] = min(e0 + s, d) * rs;
                r = make_int4(static_cast<int>(static_cast<uint32_t>(d * rs) | (static_cast<uint32_t>(o[0]) << 16)),
                              static_cast<int>(static_cast<uint32_t>(o[1]) | (static_cast<uint32_t>(o[2]) << 16)), o[3],
                              (d << 16) | e0);
                break;
            }
            base += nq;
        }
        desc[u] = r;
    }
    __syncthreads();
    const float qmax = *sinv;
    int e2 = 0;
    if (qmax > 0.f) frexpf(qmax, &e2);
    const int sq = (qmax > 0.f) ? 14 - e2 : 0;
    const float sc = ldexpf(1.f, sq);
    for (int i = threadIdx.x; i < nks * NT * 32; i += blockDim.x) {
        const int lane = i & 31, tile = i >> 5, nt = tile % NT, kk = tile / NT;
        const int bc = 8 * nt + (lane >> 2);
        const int4 dsc = desc[4 * kk + (lane & 3)];
        float v[4] = {0.f, 0.f, 0.f, 0.f};
        if (dsc.w >= 0 && bc < A2) {
            const int d = dsc.w >> 16, e0 = dsc.w & 0xffff;
#pragma unroll
            for (int s = 0; s < 4; ++s)
                if (e0 + s <= d) v[s] = g_qq[pair_index(d, e0 + s) * A2 + bc] * sc;
        }
        uint32_t h01, l01, h23, l23;
        split_f16x2(v[0], v[1], h01, l01);
        split_f16x2(v[2], v[3], h23, l23);
        *reinterpret_cast<uint4*>(tq + 4 * i) = make_uint4(h01, h23, l01, l23);
    }
    __syncthreads();
    if (threadIdx.x == 0) *sinv = ldexpf(1.f, -sq);
    __syncthreads();
}

// D (16 x 8, FP32) += A (16 x 16) B (16 x 8), FP16 operands
__device__ __forceinline__ void mma_f16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The quadratic part of V for the warp's 32 records, by the tensor cores: records are the MMA
// rows (m-tile mt, row g / g + 8 = the record of lane 16 mt + g / 16 mt + 8 + g; a lane's
// fragment rows are g = lane / 4 and g + 8), the pair slots
// of four quadruples one k-step, the surface pairs the columns.  Each lane forms the products
// q_d q_e of its four rows' records from shared memory (rec[r] = record 2 mt + half's q at its
// bead, mode 0), split into FP16 hi and lo; three MMAs per tile (hi hi, hi lo, lo hi) give about
// 22 bits.  Returns, in vq, this lane's own record's quadratic terms (already unscaled).
template <int A>
__device__ __forceinline__ void tcq_quadratic(const uint32_t* __restrict__ tq, int nks, const float* __restrict__ sq,
                                              const int (&rec)[4], int lane, float (&vq)[npair(A)]) {
    constexpr int A2 = npair(A);
    constexpr int NT = tcq_ntiles(A);
    const int4* desc = reinterpret_cast<const int4*>(tq + nks * NT * 128);
    const float sinv = *reinterpret_cast<const float*>(desc + 4 * nks);
    float acc[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.f;
    for (int kk = 0; kk < nks; ++kk) {
        const int4 dsc = desc[4 * kk + (lane & 3)];
        const uint32_t ux = static_cast<uint32_t>(dsc.x), uy = static_cast<uint32_t>(dsc.y);
        const int od = ux & 0xffffu, o0 = ux >> 16, o1 = uy & 0xffffu, o2 = uy >> 16, o3 = dsc.z;
        uint32_t ah[2][4], al[2][4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float* qb = sq + rec[r];
            const float qd = qb[od];
            uint32_t h01, l01, h23, l23;
            split_f16x2(qd * qb[o0], qd * qb[o1], h01, l01);
            split_f16x2(qd * qb[o2], qd * qb[o3], h23, l23);
            const int mt = r >> 1, hf = r & 1;
            ah[mt][hf] = h01; ah[mt][2 + hf] = h23;
            al[mt][hf] = l01; al[mt][2 + hf] = l23;
        }
        uint4 b[NT];
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) b[nt] = *reinterpret_cast<const uint4*>(tq + 4 * ((kk * NT + nt) * 32 + lane));
        // the three passes outermost, so consecutive MMAs update different tiles
#pragma unroll
        for (int pass = 0; pass < 3; ++pass)
#pragma unroll
            for (int nt = 0; nt < NT; ++nt)
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) {
                    if (pass == 0) mma_f16_16816(acc[mt][nt], ah[mt], b[nt].x, b[nt].y);
                    else if (pass == 1) mma_f16_16816(acc[mt][nt], ah[mt], b[nt].z, b[nt].w);
                    else mma_f16_16816(acc[mt][nt], al[mt], b[nt].x, b[nt].y);
                }
    }
    // D[row][col] of tile (mt, nt) sits in lane 4 (row % 8) + col % 8 / 2, register 2 (row / 8) +
    // col % 2: this lane's record (mt = lane / 16, row half = lane / 8 % 2, row = lane % 8) reads
    // its columns from the four lanes 4 (lane % 8) + t
    const int pick = lane >> 3, src = 4 * (lane & 7);
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
        for (int tp = 0; tp < 4; ++tp)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int bc = 8 * nt + 2 * tp + e;
                if (bc >= A2) continue;
                const float s0 = __shfl_sync(0xffffffffu, acc[0][nt][e], src + tp);
                const float s1 = __shfl_sync(0xffffffffu, acc[0][nt][2 + e], src + tp);
                const float s2 = __shfl_sync(0xffffffffu, acc[1][nt][e], src + tp);
                const float s3 = __shfl_sync(0xffffffffu, acc[1][nt][2 + e], src + tp);
                vq[bc] = sinv * (pick == 0 ? s0 : pick == 1 ? s1 : pick == 2 ? s2 : s3);
            }
}

// kTcq: the instantiation with the tensor-core quadratic (launched when args.tcq is set); the
// other keeps the FP32 pair loop and none of the quadratic's registers.
template <int A, int K, int QM, typename T, bool kTcq = false>
__global__ void __launch_bounds__(kThreads) pimc_fused_kernel(const FusedArgs args) {
    constexpr int A2 = npair(A);
    constexpr int A2P = (A2 + 3) / 4 * 4;
    constexpr int KP = (K + 1 + 3) / 4 * 4;
    constexpr int AP = (A + 3) / 4 * 4;
    constexpr int MR = 2 * KP + 2 * AP + 4 + A2P;
    constexpr bool kLo = (QM == kQ64) && (sizeof(T) == 4);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);

    const pbr_model& m = args.m;
    const int N = m.N, P = m.P, nfill = m.n_fill_rho, rs = args.rs;
    const int G = args.G, C = args.C, S = args.S;
    const SmemPlan plan(A, K, QM, static_cast<int>(sizeof(T)), N, P, S, args.qstride, kTcq ? 1 : 0);
    T* s_c = sm + plan.c;    T* s_e = sm + plan.e;    T* s_qq = sm + plan.qq;
    T* s_rc = sm + plan.rc;  T* s_rec = sm + plan.rec;

    // ---- model tables -> shared memory (once per CTA; the grid is persistent) -----------------
    {
        const T* g_cs = static_cast<const T*>(m.vib_cs);  const T* g_th = static_cast<const T*>(m.vib_th);
        const T* g_c = static_cast<const T*>(m.vib_c);    const T* g_d = static_cast<const T*>(m.vib_d);
        const T* g_e = static_cast<const T*>(m.vib_e);    const T* g_l = static_cast<const T*>(m.vib_l);
        const T* g_qq = static_cast<const T*>(m.vib_qq);
        const T* g_rcs = static_cast<const T*>(m.rho_cs); const T* g_rth = static_cast<const T*>(m.rho_th);
        const T* g_rc = static_cast<const T*>(m.rho_c);   const T* g_rd = static_cast<const T*>(m.rho_d);
        for (int i = threadIdx.x; i < (K + 1) * A; i += blockDim.x) s_c[i] = g_c[i];
        for (int i = threadIdx.x; i < A2P; i += blockDim.x) s_e[i] = (i < A2) ? g_e[i] : T(0);
        const int N2 = npair(N);
        if constexpr (kTcq) {
            tcq_tables<A>(reinterpret_cast<const float*>(g_qq), N, rs, plan.tcq_k,
                          reinterpret_cast<uint32_t*>(s_qq));
        } else {
            for (int i = threadIdx.x; i < N2 * A2P; i += blockDim.x) {
                const int row = i / A2P, col = i - row * A2P;
                s_qq[i] = (col < A2) ? g_qq[row * A2 + col] : T(0);
            }
        }
        for (int i = threadIdx.x; i < A; i += blockDim.x) s_rc[i] = (i < nfill) ? g_rc[i] : T(0);
        for (int i = threadIdx.x; i < N * MR; i += blockDim.x) {
            const int j = i / MR, o = i - j * MR;
            T v = T(0);
            if (o < KP) { if (o <= K) v = g_cs[o * N + j]; }
            else if (o < 2 * KP) { if (o - KP <= K) v = g_th[(o - KP) * N + j]; }
            else if (o < 2 * KP + AP) { const int a = o - 2 * KP; if (a < A) v = g_d[a * N + j]; }
            else if (o < 2 * KP + 2 * AP) { const int a = o - 2 * KP - AP; if (a < nfill) v = g_rd[a * N + j]; }
            else if (o == 2 * KP + 2 * AP) v = g_rcs[j];
            else if (o == 2 * KP + 2 * AP + 1) v = g_rth[j];
            else if (o >= 2 * KP + 2 * AP + 4) { const int pr = o - 2 * KP - 2 * AP - 4; if (pr < A2) v = g_l[j * A2 + pr]; }
            s_rec[i] = v;
        }
    }
    __syncthreads();

    const int tid = threadIdx.x;
    const int grp = tid >> args.logG;
    const int g = tid & (G - 1);
    const int lane = tid & 31;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    T* qs = sm + plan.q + grp * args.qstride;
    T* ql = kLo ? (sm + plan.qlo + grp * args.qstride) : nullptr;
    const int p_begin = g * C;
    const int p_end = min(P, p_begin + C);
    const T tau_l2 = T(m.tau * 1.4426950408889634);   // tau * log2(e)

    for (int64_t base = static_cast<int64_t>(blockIdx.x) * S; base < args.X;
         base += static_cast<int64_t>(gridDim.x) * S) {
        const int64_t sidx = base + grp;
        const bool active = sidx < args.X;

        // ============================ phase A: q into shared memory ============================
        if (active) {
            const int NP = N * P;
            if (QM == kSample) {
                const int src = draw_sample_smem<T>(m, qs, rs, sidx, args.offset, args.key0,
                                                    args.key1, g, G, gmask);
                if (args.out.src_out && g == 0) args.out.src_out[sidx] = src;
                if (args.out.q_out) {
                    float* qo = args.out.q_out + sidx * static_cast<int64_t>(NP);
                    for (int i = g; i < NP; i += G) {
                        const int j = i / P, p = i - j * P;
                        qo[i] = static_cast<float>(qs[qidx(j, p, rs)]);
                    }
                }
            } else if (QM == kQ64) {
                const double* qin = static_cast<const double*>(args.q_in) + sidx * static_cast<int64_t>(NP);
                for (int i = g; i < NP; i += G) {
                    const int j = i / P, p = i - j * P;
                    const double v = qin[i];
                    const T hi = T(v);
                    qs[qidx(j, p, rs)] = hi;
                    if (kLo) ql[qidx(j, p, rs)] = T(v - static_cast<double>(hi));
                }
                __syncwarp(gmask);
            } else {
                const float* qin = static_cast<const float*>(args.q_in) + sidx * static_cast<int64_t>(NP);
                for (int i = g; i < NP; i += G) {
                    const int j = i / P, p = i - j * P;
                    qs[qidx(j, p, rs)] = T(qin[i]);
                }
                __syncwarp(gmask);
            }
        }

        // ============================ phase B: the thread's bead chunk ==========================
        T nser[K + 1][A][A];
#pragma unroll
        for (int k = 0; k <= K; ++k)
#pragma unroll
            for (int r = 0; r < A; ++r)
#pragma unroll
                for (int c = 0; c < A; ++c) nser[k][r][c] = (k == 0 && r == c) ? T(1) : T(0);
        int nexp = 0;
        LogSum<T> lrho[A];
        LogSum<T> lsum;
        T uw[A][A];          // eigenvectors of the previous bead: warm start of the next Jacobi

        // One bead step of the chunk: bead p of the chunk (step ii), on = this lane's record is
        // live.  Run by every lane for ii < C (the warp-wide tensor-core quadratic needs all 32
        // records in step) in the tensor-core instantiation, and at 3 surfaces, where the uniform
        // loop measured 17 % faster (A = 3, N = 8, P = 48); else only by live lanes over their own
        // beads.
        auto bead = [&](const int ii, const int p, const bool on) {
            const int ip = qidx(0, p, rs);
            T v[A2P], osr[K + 1][A];
            T qmax = T(0);
            if (on) {
                const int pn = (p + 1 == P) ? 0 : p + 1;
                const int ipn = qidx(0, pn, rs);
                // ---- O-matrix exponents and the linear part of V, one pass over the modes ----
                T phv[K + 1][A], phr[A];
#pragma unroll
                for (int k = 0; k <= K; ++k)
#pragma unroll
                    for (int a = 0; a < A; ++a) phv[k][a] = s_c[k * A + a];
#pragma unroll
                for (int a = 0; a < A; ++a) phr[a] = s_rc[a];
                ldv(s_e, v);
                T dsum[K + 1];
#pragma unroll
                for (int k = 0; k <= K; ++k) dsum[k] = T(0);
                T rdsum = T(0);
                for (int j = 0; j < N; ++j) {
                    const T* rec = s_rec + j * MR;
                    T cs[KP], th[KP], dv[AP], rdv[AP], rx[4], lr[A2P];
                    ldv(rec, cs);
                    ldv(rec + KP, th);
                    ldv(rec + 2 * KP, dv);
                    ldv(rec + 2 * KP + AP, rdv);
                    ldv(rec + 2 * KP + 2 * AP, rx);
                    ldv(rec + 2 * KP + 2 * AP + 4, lr);
                    const T qa = qs[ip + j * rs], qb = qs[ipn + j * rs];
                    if constexpr (kTcq) qmax = max(qmax, dev_fabs(qa));
                    T dq = qa - qb;
                    if (kLo) dq += ql[ip + j * rs] - ql[ipn + j * rs];
                    const T dq2 = dq * dq;
#pragma unroll
                    for (int k = 0; k <= K; ++k) dsum[k] = fma(cs[k], dq2, dsum[k]);
                    rdsum = fma(rx[0], dq2, rdsum);
#pragma unroll
                    for (int a = 0; a < A; ++a) {
                        const T ua = qa - dv[a], ub = qb - dv[a];
                        const T sq = fma(ua, ua, ub * ub);
#pragma unroll
                        for (int k = 0; k <= K; ++k) phv[k][a] = fma(-th[k], sq, phv[k][a]);
                        if (a < nfill) {
                            const T ra = qa - rdv[a], rb = qb - rdv[a];
                            phr[a] = fma(-rx[1], fma(ra, ra, rb * rb), phr[a]);
                        }
                    }
#pragma unroll
                    for (int pr = 0; pr < A2; ++pr) v[pr] = fma(lr[pr], qa, v[pr]);
                }
#pragma unroll
                for (int a = 0; a < A; ++a) {
#pragma unroll
                    for (int k = 0; k <= K; ++k) phv[k][a] -= dsum[k];
                    phr[a] -= rdsum;
                }
                // ---- S12 and the scaled O series ----
                T lmax = phv[0][0];
#pragma unroll
                for (int a = 1; a < A; ++a) lmax = max(lmax, phv[0][a]);
#pragma unroll
                for (int a = 0; a < A; ++a)
                    if (a < nfill) lmax = max(lmax, phr[a]);
                lsum.add(lmax);
#pragma unroll
                for (int a = 0; a < A; ++a)
                    if (a < nfill) lrho[a].add(phr[a] - lmax);
#pragma unroll
                for (int a = 0; a < A; ++a) {
                    T ek[K + 1];
                    ek[0] = T(1);
#pragma unroll
                    for (int k = 1; k <= K; ++k) {
                        T acc = T(0);
#pragma unroll
                        for (int i = 1; i <= k; ++i) acc = fma(T(i) * phv[i][a], ek[k - i], acc);
                        ek[k] = acc * (T(1) / T(k));
                    }
                    const T e0 = dev_exp<T>(phv[0][a] - lmax);
#pragma unroll
                    for (int k = 0; k <= K; ++k) osr[k][a] = e0 * ek[k];
                }
            }
            // ---- quadratic part of V ----
            bool quad_done = false;
            if constexpr (kTcq) {
                {
                    // tensor cores, unless a record of the warp has a coordinate beyond FP16's
                    // range for the products (then the FP32 loop below over the global table)
                    if (!__any_sync(0xffffffffu, on && !(qmax <= T(kTcqMaxQ)))) {
                        int rec[4];
                        const int wb = tid & ~31;
#pragma unroll
                        for (int r = 0; r < 4; ++r) {
                            const int l2 = wb + 16 * (r >> 1) + 8 * (r & 1) + (lane >> 2);   // fragment rows: lane / 4 (+ 8)
                            const int pb = min((l2 & (G - 1)) * C + ii, P - 1);
                            rec[r] = plan.q + (l2 >> args.logG) * args.qstride + qidx(0, pb, rs);
                        }
                        float vq[A2];
                        tcq_quadratic<A>(reinterpret_cast<const uint32_t*>(s_qq), plan.tcq_k,
                                         reinterpret_cast<const float*>(sm), rec, lane, vq);
#pragma unroll
                        for (int pr = 0; pr < A2; ++pr) v[pr] += vq[pr];
                    } else if (on) {
                        const float* gq = static_cast<const float*>(m.vib_qq);
                        const int N2 = npair(N);
                        int od = 0, oe = 0;
                        for (int row = 0; row < N2; ++row) {
                            const T w = qs[ip + od] * qs[ip + oe];
#pragma unroll
                            for (int pr = 0; pr < A2; ++pr) v[pr] = fma(__ldg(gq + row * A2 + pr), w, v[pr]);
                            const bool wrap = (oe == od);
                            od = wrap ? od + rs : od;
                            oe = wrap ? 0 : oe + rs;
                        }
                    }
                    quad_done = true;
                }
            }
            if (on && !quad_done) {
                // one flat loop over the mode pairs (d, e <= d) in table order, unrolled so
                // several pairs' loads are in flight together
                if constexpr (A >= kFlatPairsMinA) {
                    const int N2 = npair(N);
                    int od = 0, oe = 0;                  // offsets d * rs, e * rs of the pair (d, e)
#pragma unroll 4
                    for (int row = 0; row < N2; ++row) {
                        const T w = qs[ip + od] * qs[ip + oe];
                        T qrow[A2P];
                        ldv(s_qq + row * A2P, qrow);
#pragma unroll
                        for (int pr = 0; pr < A2; ++pr) v[pr] = fma(qrow[pr], w, v[pr]);
                        const bool wrap = (oe == od);        // e == d: next row starts (d + 1, 0)
                        od = wrap ? od + rs : od;
                        oe = wrap ? 0 : oe + rs;
                    }
                } else {
                    int row = 0;
                    for (int d = 0; d < N; ++d) {
                        const T qd = qs[ip + d * rs];
                        for (int e = 0; e <= d; ++e, ++row) {
                            const T w = qd * qs[ip + e * rs];
                            T qrow[A2P];
                            ldv(s_qq + row * A2P, qrow);
#pragma unroll
                            for (int pr = 0; pr < A2; ++pr) v[pr] = fma(qrow[pr], w, v[pr]);
                        }
                    }
                }
            }
            if (on) {
                // ---- M = exp(-tau V): scaling and squaring in FP32, Jacobi (warm-started from the
                //      previous bead) in the FP64 validation build ----
                T M[A][A];
                if constexpr (sizeof(T) == 4 && A >= kExpmMinA) {
                    float vp[npair(A)];
#pragma unroll
                    for (int i = 0; i < npair(A); ++i) vp[i] = v[i];
                    nexp += expm_neg_tau<A>(vp, static_cast<float>(m.tau), M);
                } else {
                    const bool cold = ((p - p_begin) & 7) == 0;   // fresh basis every 8 beads
                    if (cold) {
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c < A; ++c) uw[r][c] = (r == c) ? T(1) : T(0);
                    }
                    T am[A][A];
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c <= b; ++c) { am[b][c] = v[pair_index(b, c)]; am[c][b] = am[b][c]; }
                    if (!cold) {
                        // am <- U^T V U in the previous bead's eigenbasis
                        T w[A][A];
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(am[r][mm], uw[mm][c], acc);
                                w[r][c] = acc;
                            }
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c <= r; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(uw[mm][r], w[mm][c], acc);
                                am[r][c] = acc;
                                am[c][r] = acc;
                            }
                    }
                    jacobi_accumulate<T, A>(am, uw, sizeof(T) == 4 ? 10 : 16);
                    T t[A];
                    T tmax = -tau_l2 * am[0][0];
#pragma unroll
                    for (int i = 0; i < A; ++i) { t[i] = -tau_l2 * am[i][i]; tmax = max(tmax, t[i]); }
                    const int n2 = static_cast<int>(floor(tmax));
                    nexp += n2;
                    T ev[A];
#pragma unroll
                    for (int i = 0; i < A; ++i) ev[i] = dev_exp2<T>(t[i] - T(n2));
#pragma unroll
                    for (int r = 0; r < A; ++r)
#pragma unroll
                        for (int c = 0; c <= r; ++c) {
                            T acc = T(0);
#pragma unroll
                            for (int i = 0; i < A; ++i) acc = fma(uw[r][i] * ev[i], uw[c][i], acc);
                            M[r][c] = acc;
                            M[c][r] = acc;
                        }
                }
                // ---- ring update N(h) <- N(h) M diag(O(h)) ----
                if (p == p_begin) {
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c < A; ++c) nser[k][r][c] = M[r][c] * osr[k][c];
                } else {
#pragma unroll
                    for (int r = 0; r < A; ++r) {
                        T y[K + 1][A];
#pragma unroll
                        for (int i = 0; i <= K; ++i)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(nser[i][r][mm], M[mm][c], acc);
                                y[i][c] = acc;
                            }
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int i = 0; i <= k; ++i) acc = fma(y[i][c], osr[k - i][c], acc);
                                nser[k][r][c] = acc;
                            }
                    }
                }
                nexp += renormalise<T, K, A>(nser);
            }
        };
        if constexpr (kTcq || A == 3) {
            if constexpr (kTcq) __syncwarp();  // the quadratic reads the q of every sample of the warp
            for (int ii = 0; ii < C; ++ii) bead(ii, p_begin + ii, active && p_begin + ii < p_end);
        } else {
            if (active)
                for (int p = p_begin; p < p_end; ++p) bead(p - p_begin, p, true);
        }

        // ============================ phase C: combine the chunks ===============================
        for (int st = 1; st < G; st <<= 1) {
            T oth[K + 1][A][A];
#pragma unroll
            for (int k = 0; k <= K; ++k)
#pragma unroll
                for (int r = 0; r < A; ++r)
#pragma unroll
                    for (int c = 0; c < A; ++c) oth[k][r][c] = __shfl_down_sync(0xffffffffu, nser[k][r][c], st, G);
            const int oexp = __shfl_down_sync(0xffffffffu, nexp, st, G);
            if ((g & (2 * st - 1)) == 0 && g + st < G) {
#pragma unroll
                for (int r = 0; r < A; ++r) {
                    T z[K + 1][A];
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) {
                            T acc = T(0);
#pragma unroll
                            for (int i = 0; i <= k; ++i)
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(nser[i][r][mm], oth[k - i][mm][c], acc);
                            z[k][c] = acc;
                        }
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) nser[k][r][c] = z[k][c];
                }
                nexp += oexp;
                nexp += renormalise<T, K, A>(nser);
            }
        }
        // the chunks' log sums, compensated (FP32 pairs in the FP32 build), summed down to g = 0
        for (int st = G >> 1; st >= 1; st >>= 1) {
#pragma unroll
            for (int a = 0; a < A; ++a) lrho[a].merge(lrho[a].shfl_down(st, G));
            lsum.merge(lsum.shfl_down(st, G));
        }
        double lr_d[A];
#pragma unroll
        for (int a = 0; a < A; ++a) lr_d[a] = lrho[a].value();
        const double ls_d = lsum.value();

        // ============================ phase D: outputs ==========================================
        if (active && g == 0) {
            // traces summed in T: each diagonal entry already carries T's rounding, which a wider
            // sum would not remove; one conversion per coefficient
            double coef[K + 1];
#pragma unroll
            for (int k = 0; k <= K; ++k) {
                T tr = T(0);
#pragma unroll
                for (int r = 0; r < A; ++r) tr += nser[k][r][r];
                coef[k] = scale_pow2(static_cast<double>(tr), nexp);
            }
            double rho = 0.0;
#pragma unroll
            for (int a = 0; a < A; ++a)
                if (a < nfill) rho += exp_out<T>(lr_d[a]);
            const pbr_outputs& o = args.out;
            o.s_rho[sidx] = rho;
            o.s_g[sidx] = coef[0];
            bool bad = !isfinite(rho) || !isfinite(coef[0]);
            if (K > 0) {
                const double db = m.delta_beta;
                double gp = 0.0, gm = 0.0;
#pragma unroll
                for (int k = K; k >= 0; --k) { gp = gp * db + coef[k]; gm = gm * (-db) + coef[k]; }
                if (o.s_gp) o.s_gp[sidx] = gp;
                if (o.s_gm) o.s_gm[sidx] = gm;
                bad = bad || !isfinite(gp) || !isfinite(gm);
            }
            if (o.g_coef) {
#pragma unroll
                for (int k = 0; k <= K; ++k) o.g_coef[sidx * (K + 1) + k] = coef[k];
            }
            if (o.log_scale) o.log_scale[sidx] = ls_d + static_cast<double>(P) * m.log_c0;
            if (bad) flag_status(o.status, PBR_ERR_NONFINITE);
        }
        __syncwarp();
    }
}

// Sampler only: q [X, N, P] (FP32) and the source surfaces, the reference's draw_sample +
// transform_sampled_coordinates (pimc.py:326-334, 613-631).
template <typename T>
__global__ void __launch_bounds__(kThreads) sample_q_kernel(const FusedArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const pbr_model& m = args.m;
    const int N = m.N, P = m.P, G = args.G, S = args.S, rs = args.rs;
    const int tid = threadIdx.x, grp = tid >> args.logG, g = tid & (G - 1), lane = tid & 31;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    T* qs = reinterpret_cast<T*>(smem_raw) + grp * args.qstride;
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * S; base < args.X;
         base += static_cast<int64_t>(gridDim.x) * S) {
        const int64_t sidx = base + grp;
        if (sidx < args.X) {
            const int src = draw_sample_smem<T>(m, qs, rs, sidx, args.offset, args.key0, args.key1,
                                                g, G, gmask);
            if (args.out.src_out && g == 0) args.out.src_out[sidx] = src;
            const int NP = N * P;
            float* qo = args.out.q_out + sidx * static_cast<int64_t>(NP);
            int j = g / P, p = g - j * P;                     // element i = j P + p, stepped by G
            for (int i = g; i < NP; i += G) {
                qo[i] = static_cast<float>(qs[qidx(j, p, rs)]);
                for (p += G; p >= P; p -= P) ++j;
            }
        }
        __syncwarp();
    }
}

// Sampling only, streamed to global memory for any N x P: a warp draws mode j of 32 consecutive
// samples (lane = sample, so the ring-factor coefficients are broadcast loads), buffers 32 beads
// per lane in shared memory and writes them back as 128-byte rows of q [X][N][P].
constexpr int kRowsWarps = 8;
template <typename T>
__global__ void __launch_bounds__(kRowsWarps * 32) sample_q_rows_kernel(const FusedArgs args) {
    __shared__ float buf[kRowsWarps][32][33];
    const pbr_model& m = args.m;
    const int N = m.N, P = m.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t groups = (args.X + 31) / 32;
    float (*wb)[33] = buf[warp];
    for (int64_t wg = static_cast<int64_t>(blockIdx.x) * kRowsWarps + warp; wg < groups * N;
         wg += static_cast<int64_t>(gridDim.x) * kRowsWarps) {
        const int j = static_cast<int>(wg % N);
        const int64_t xb = (wg / N) * 32;
        const int64_t x = xb + lane;
        const bool valid = x < args.X;
        const uint64_t sg = args.offset + static_cast<uint64_t>(valid ? x : xb);
        const int src = draw_source<T>(m, sg, args.key0, args.key1);
        if (valid && j == 0 && args.out.src_out) args.out.src_out[x] = src;
        const T dsh = static_cast<const T*>(m.rho_d)[static_cast<int64_t>(src) * N + j];
        draw_mode_chain_to<T>(m, j, sg, args.key0, args.key1, dsh, [&](int p, T v) {
            wb[lane][p & 31] = static_cast<float>(v);
            if ((p & 31) == 0) {                       // beads p .. p+31 of the 32 rows are complete
                __syncwarp();
                const int pe = min(P, p + 32);
                for (int i = 0; i < 32; ++i) {
                    const int64_t xi = xb + i;
                    if (xi < args.X && p + lane < pe)
                        args.out.q_out[(xi * N + j) * static_cast<int64_t>(P) + p + lane] = wb[i][lane];
                }
                __syncwarp();
            }
        });
    }
}

// host-side launcher, instantiated per surface count in pbr_fused_a*.cu
template <int A>
int launch_fused(int K, int qmode, int precision, const FusedArgs& args, cudaStream_t stream);

}  // namespace pbr
