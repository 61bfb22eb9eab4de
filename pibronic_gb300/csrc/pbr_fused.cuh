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
//            (phi^rho_pa - ln S12_p)), all in FP64 with the accumulated power-of-two exponent.
#pragma once

#include "pbr_common.cuh"

namespace pbr {

constexpr int kThreads = 128;
constexpr int kMaxChunk = 8;       // beads per thread on the sampling path
enum QMode : int { kSample = 0, kQ64 = 1, kQ32 = 2 };

struct FusedArgs {
    pbr_model m;
    const void* q_in;
    int64_t X;
    pbr_outputs out;
    uint32_t key0, key1;
    uint64_t offset;
    int G, logG, C, S;
    int a2p;        // padded row length of the packed quadratic table in shared memory
    int qstride;    // elements per sample in the q region
};

__host__ __device__ inline int align_up(int x, int a) { return (x + a - 1) / a * a; }

// Shared-memory plan (in elements of the table type, esz bytes each); identical on host and device.
struct SmemPlan {
    int cs, th, c, d, e, l, qq, rcs, rth, rc, rd, trig, q, qlo, total_bytes;
    __host__ __device__ SmemPlan(int A, int K, int qm, int esz, int N, int P, int a2p, int S,
                                 int qstride) {
        const int A2 = npair(A);
        const int N2 = npair(N);
        int o = 0;
        auto take = [&](int n) { int r = o; o = align_up(o + n, 4); return r; };
        cs = take((K + 1) * N); th = take((K + 1) * N); c = take((K + 1) * A); d = take(A * N);
        e = take(A2); l = take(N * A2); qq = take(N2 * a2p);
        rcs = take(N); rth = take(N); rc = take(A); rd = take(A * N);
        trig = take(qm == kSample ? 2 * P : 0);
        q = take(S * qstride);
        qlo = take((qm == kQ64 && esz == 4) ? S * qstride : 0);
        total_bytes = o * esz;
    }
};

template <typename T> __device__ __forceinline__ T dev_fabs(T x) { return x < T(0) ? -x : x; }

// Phase A on the sampling path: the G threads of one sample (lanes gmask) draw the source surface
// and the normal-mode coordinates and transform them to bead coordinates q[j][p] in shared
// memory (row stride P).  Returns the source surface.  pimc.py:326-334, 386-389, 613-631.
template <typename T>
__device__ int draw_sample_smem(const pbr_model& m, const T* s_trig, T* qs, int64_t sidx,
                                uint64_t offset, uint32_t key0, uint32_t key1, int g, int G, int C,
                                int p_begin, unsigned gmask) {
    const int N = m.N, P = m.P;
    const uint64_t sg = offset + static_cast<uint64_t>(sidx);
    const uint32_t lo = static_cast<uint32_t>(sg), hi = static_cast<uint32_t>(sg >> 32);
    // source surface ~ Categorical(state weights) (pimc.py:386-389)
    const u32x4 rs = philox4x32_10(u32x4{0xFFFFFFFFu, lo, hi, 1u}, key0, key1);
    const float us = u01(rs.x);
    const T* cdf = static_cast<const T*>(m.src_cdf);
    int src = 0;
    for (int a = 0; a < m.A_rho - 1; ++a) src += (us >= static_cast<float>(cdf[a])) ? 1 : 0;
    // normal-mode coordinates cc[j][s] ~ Normal(0, std[src][j][s]) (pimc.py:326-334)
    const T* stdp = static_cast<const T*>(m.mode_std) + static_cast<int64_t>(src) * N * P;
    const int NP = N * P;
    const int ncalls = (NP + 3) >> 2;
    for (int cidx = g; cidx < ncalls; cidx += G) {
        const u32x4 r = philox4x32_10(u32x4{static_cast<uint32_t>(cidx), lo, hi, 0u}, key0, key1);
        float z[4];
        box_muller(r.x, r.y, z[0], z[1]);
        box_muller(r.z, r.w, z[2], z[3]);
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int i = 4 * cidx + t;
            if (i < NP) qs[i] = T(z[t]) * stdp[i];
        }
    }
    __syncwarp(gmask);
    // ring transform q_p = sum_s B_ps cc_s + d^rho_src (pimc.py:618-624), in place per mode block
    const T inv_sqrt_p = T(1.0 / sqrt(static_cast<double>(P)));
    const int kmax = (P - 1) / 2;
    const bool even = (P % 2) == 0;
    const T* dsrc = static_cast<const T*>(m.rho_d) + static_cast<int64_t>(src) * N;
    constexpr int JB = 4;
    for (int j0 = 0; j0 < N; j0 += JB) {
        T acc[kMaxChunk][JB];
#pragma unroll
        for (int b = 0; b < kMaxChunk; ++b) {
            const int p = p_begin + b;
#pragma unroll
            for (int jj = 0; jj < JB; ++jj) {
                const int j = min(j0 + jj, N - 1);
                T v = qs[j * P] * inv_sqrt_p;
                if (even) v += ((p & 1) ? -qs[j * P + P - 1] : qs[j * P + P - 1]) * inv_sqrt_p;
                acc[b][jj] = v;
            }
        }
        int mm[kMaxChunk];
#pragma unroll
        for (int b = 0; b < kMaxChunk; ++b) mm[b] = 0;
        for (int k = 1; k <= kmax; ++k) {
            T cc_c[JB], cc_s[JB];
#pragma unroll
            for (int jj = 0; jj < JB; ++jj) {
                const int j = min(j0 + jj, N - 1);
                cc_c[jj] = qs[j * P + 2 * k - 1];
                cc_s[jj] = qs[j * P + 2 * k];
            }
#pragma unroll
            for (int b = 0; b < kMaxChunk; ++b) {
                const int p = p_begin + b;
                int mb = mm[b] + p;                    // (k p) mod P, incremental
                mb = (mb >= P) ? mb - P : mb;
                mb = (mb >= P) ? mb % P : mb;
                mm[b] = mb;
                const T cth = s_trig[2 * mb], sth = s_trig[2 * mb + 1];
#pragma unroll
                for (int jj = 0; jj < JB; ++jj) acc[b][jj] += cc_c[jj] * cth + cc_s[jj] * sth;
            }
        }
        __syncwarp(gmask);
#pragma unroll
        for (int b = 0; b < kMaxChunk; ++b) {
            const int p = p_begin + b;
            if (b < C && p < P) {
#pragma unroll
                for (int jj = 0; jj < JB; ++jj) {
                    const int j = j0 + jj;
                    if (j < N) qs[j * P + p] = acc[b][jj] + dsrc[j];
                }
            }
        }
        __syncwarp(gmask);
    }
    return src;
}

// Fill the sampling-path trig table: trig[2m], trig[2m+1] = sqrt(2/P) (cos, sin)(2 pi m / P).
template <typename T>
__device__ void fill_trig(T* s_trig, int P) {
    const double amp = sqrt(2.0 / P);
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        double s, c;
        sincospi(2.0 * i / P, &s, &c);
        s_trig[2 * i] = T(amp * c);
        s_trig[2 * i + 1] = T(amp * s);
    }
}

template <int A, int K, int QM, typename T>
__global__ void __launch_bounds__(kThreads) pimc_fused_kernel(const FusedArgs args) {
    constexpr int A2 = npair(A);
    constexpr bool kLo = (QM == kQ64) && (sizeof(T) == 4);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);

    const pbr_model& m = args.m;
    const int N = m.N, P = m.P, nfill = m.n_fill_rho;
    const int G = args.G, C = args.C, S = args.S;
    const SmemPlan plan(A, K, QM, static_cast<int>(sizeof(T)), N, P, args.a2p, S, args.qstride);
    T* s_cs = sm + plan.cs;  T* s_th = sm + plan.th;  T* s_c = sm + plan.c;  T* s_d = sm + plan.d;
    T* s_e = sm + plan.e;    T* s_l = sm + plan.l;    T* s_qq = sm + plan.qq;
    T* s_rcs = sm + plan.rcs; T* s_rth = sm + plan.rth; T* s_rc = sm + plan.rc; T* s_rd = sm + plan.rd;
    T* s_trig = sm + plan.trig;

    // ---- model tables -> shared memory (once per CTA; the grid is persistent) -----------------
    {
        const T* g_cs = static_cast<const T*>(m.vib_cs);  const T* g_th = static_cast<const T*>(m.vib_th);
        const T* g_c = static_cast<const T*>(m.vib_c);    const T* g_d = static_cast<const T*>(m.vib_d);
        const T* g_e = static_cast<const T*>(m.vib_e);    const T* g_l = static_cast<const T*>(m.vib_l);
        const T* g_qq = static_cast<const T*>(m.vib_qq);
        const T* g_rcs = static_cast<const T*>(m.rho_cs); const T* g_rth = static_cast<const T*>(m.rho_th);
        const T* g_rc = static_cast<const T*>(m.rho_c);   const T* g_rd = static_cast<const T*>(m.rho_d);
        for (int i = threadIdx.x; i < (K + 1) * N; i += blockDim.x) { s_cs[i] = g_cs[i]; s_th[i] = g_th[i]; }
        for (int i = threadIdx.x; i < (K + 1) * A; i += blockDim.x) s_c[i] = g_c[i];
        for (int i = threadIdx.x; i < A * N; i += blockDim.x) {
            s_d[i] = g_d[i];
            s_rd[i] = (i < nfill * N) ? g_rd[i] : T(0);
        }
        for (int i = threadIdx.x; i < A2; i += blockDim.x) s_e[i] = g_e[i];
        for (int i = threadIdx.x; i < N * A2; i += blockDim.x) s_l[i] = g_l[i];
        const int N2 = npair(N);
        for (int i = threadIdx.x; i < N2 * args.a2p; i += blockDim.x) {
            const int row = i / args.a2p, col = i - row * args.a2p;
            s_qq[i] = (col < A2) ? g_qq[row * A2 + col] : T(0);
        }
        for (int i = threadIdx.x; i < N; i += blockDim.x) { s_rcs[i] = g_rcs[i]; s_rth[i] = g_rth[i]; }
        for (int i = threadIdx.x; i < A; i += blockDim.x) s_rc[i] = (i < nfill) ? g_rc[i] : T(0);
        if (QM == kSample) fill_trig<T>(s_trig, P);
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
            if (QM == kSample) {
                const int src = draw_sample_smem<T>(m, s_trig, qs, sidx, args.offset, args.key0,
                                                    args.key1, g, G, C, p_begin, gmask);
                if (args.out.src_out && g == 0) args.out.src_out[sidx] = src;
                if (args.out.q_out) {
                    const int NP = N * P;
                    float* qo = args.out.q_out + sidx * static_cast<int64_t>(NP);
                    for (int i = g; i < NP; i += G) qo[i] = static_cast<float>(qs[i]);
                }
            } else {
                const int NP = N * P;
                if (QM == kQ64) {
                    const double* qin = static_cast<const double*>(args.q_in) + sidx * static_cast<int64_t>(NP);
                    for (int i = g; i < NP; i += G) {
                        const double v = qin[i];
                        const T hi = T(v);
                        qs[i] = hi;
                        if (kLo) ql[i] = T(v - static_cast<double>(hi));
                    }
                } else {
                    const float* qin = static_cast<const float*>(args.q_in) + sidx * static_cast<int64_t>(NP);
                    for (int i = g; i < NP; i += G) qs[i] = T(qin[i]);
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
        double lrho[A];
#pragma unroll
        for (int a = 0; a < A; ++a) lrho[a] = 0.0;
        double lsum = 0.0;
        bool first = true;

        if (active) {
            for (int p = p_begin; p < p_end; ++p) {
                const int pn = (p + 1 == P) ? 0 : p + 1;
                // ---- O-matrix exponents and the linear part of V, one pass over the modes ----
                T phv[K + 1][A], phr[A], v[A2];
#pragma unroll
                for (int k = 0; k <= K; ++k)
#pragma unroll
                    for (int a = 0; a < A; ++a) phv[k][a] = s_c[k * A + a];
#pragma unroll
                for (int a = 0; a < A; ++a) phr[a] = s_rc[a];
#pragma unroll
                for (int pr = 0; pr < A2; ++pr) v[pr] = s_e[pr];
                T dsum[K + 1];
#pragma unroll
                for (int k = 0; k <= K; ++k) dsum[k] = T(0);
                T rdsum = T(0);
                for (int j = 0; j < N; ++j) {
                    const T qa = qs[j * P + p], qb = qs[j * P + pn];
                    T dq = qa - qb;
                    if (kLo) dq += ql[j * P + p] - ql[j * P + pn];
                    const T dq2 = dq * dq;
#pragma unroll
                    for (int k = 0; k <= K; ++k) dsum[k] = fma(s_cs[k * N + j], dq2, dsum[k]);
                    rdsum = fma(s_rcs[j], dq2, rdsum);
#pragma unroll
                    for (int a = 0; a < A; ++a) {
                        const T da = s_d[a * N + j];
                        const T ua = qa - da, ub = qb - da;
                        const T sq = fma(ua, ua, ub * ub);
#pragma unroll
                        for (int k = 0; k <= K; ++k) phv[k][a] = fma(-s_th[k * N + j], sq, phv[k][a]);
                        if (a < nfill) {
                            const T ra = qa - s_rd[a * N + j], rb = qb - s_rd[a * N + j];
                            phr[a] = fma(-s_rth[j], fma(ra, ra, rb * rb), phr[a]);
                        }
                    }
#pragma unroll
                    for (int pr = 0; pr < A2; ++pr) v[pr] = fma(s_l[j * A2 + pr], qa, v[pr]);
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
                lsum += static_cast<double>(lmax);
#pragma unroll
                for (int a = 0; a < A; ++a)
                    if (a < nfill) lrho[a] += static_cast<double>(phr[a] - lmax);
                T osr[K + 1][A];
#pragma unroll
                for (int a = 0; a < A; ++a) {
                    T ek[K + 1];
                    ek[0] = T(1);
#pragma unroll
                    for (int k = 1; k <= K; ++k) {
                        T acc = T(0);
#pragma unroll
                        for (int i = 1; i <= k; ++i) acc = fma(T(i) * phv[i][a], ek[k - i], acc);
                        ek[k] = acc / T(k);
                    }
                    const T e0 = dev_exp<T>(phv[0][a] - lmax);
#pragma unroll
                    for (int k = 0; k <= K; ++k) osr[k][a] = e0 * ek[k];
                }
                // ---- quadratic part of V ----
                {
                    int row = 0;
                    for (int d = 0; d < N; ++d) {
                        const T qd = qs[d * P + p];
                        for (int e = 0; e <= d; ++e, ++row) {
                            const T w = qd * qs[e * P + p];
                            const T* qrow = s_qq + row * args.a2p;
#pragma unroll
                            for (int pr = 0; pr < A2; ++pr) v[pr] = fma(qrow[pr], w, v[pr]);
                        }
                    }
                }
                // ---- M = exp(-tau V) by Jacobi ----
                T M[A][A];
                {
                    T am[A][A], u[A][A];
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c <= b; ++c) { am[b][c] = v[pair_index(b, c)]; am[c][b] = am[b][c]; }
                    jacobi_eigh<T, A>(am, u, sizeof(T) == 4 ? 10 : 16);
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
                            for (int i = 0; i < A; ++i) acc = fma(u[r][i] * ev[i], u[c][i], acc);
                            M[r][c] = acc;
                            M[c][r] = acc;
                        }
                }
                // ---- ring update N(h) <- N(h) M diag(O(h)) ----
                if (first) {
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c < A; ++c) nser[k][r][c] = M[r][c] * osr[k][c];
                    first = false;
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
                // ---- power-of-two renormalisation ----
                {
                    T mx = T(0);
#pragma unroll
                    for (int r = 0; r < A; ++r)
#pragma unroll
                        for (int c = 0; c < A; ++c) mx = max(mx, dev_fabs(nser[0][r][c]));
                    if (mx > T(0) && isfinite(mx)) {
                        int e2;
                        frexp(mx, &e2);
                        const T sc = ldexp(T(1), -e2);
                        nexp += e2;
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int r = 0; r < A; ++r)
#pragma unroll
                                for (int c = 0; c < A; ++c) nser[k][r][c] *= sc;
                    }
                }
            }
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
                T mx = T(0);
#pragma unroll
                for (int r = 0; r < A; ++r)
#pragma unroll
                    for (int c = 0; c < A; ++c) mx = max(mx, dev_fabs(nser[0][r][c]));
                if (mx > T(0) && isfinite(mx)) {
                    int e2;
                    frexp(mx, &e2);
                    const T sc = ldexp(T(1), -e2);
                    nexp += e2;
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int r = 0; r < A; ++r)
#pragma unroll
                            for (int c = 0; c < A; ++c) nser[k][r][c] *= sc;
                }
            }
        }
        for (int st = G >> 1; st >= 1; st >>= 1) {
#pragma unroll
            for (int a = 0; a < A; ++a) lrho[a] += __shfl_down_sync(0xffffffffu, lrho[a], st, G);
            lsum += __shfl_down_sync(0xffffffffu, lsum, st, G);
        }

        // ============================ phase D: outputs ==========================================
        if (active && g == 0) {
            double coef[K + 1];
#pragma unroll
            for (int k = 0; k <= K; ++k) {
                double tr = 0.0;
#pragma unroll
                for (int r = 0; r < A; ++r) tr += static_cast<double>(nser[k][r][r]);
                coef[k] = ldexp(tr, nexp);
            }
            double rho = 0.0;
#pragma unroll
            for (int a = 0; a < A; ++a)
                if (a < nfill) rho += exp(lrho[a]);
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
            if (o.log_scale) o.log_scale[sidx] = lsum + static_cast<double>(P) * m.log_c0;
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
    T* s_trig = reinterpret_cast<T*>(smem_raw);
    const pbr_model& m = args.m;
    const int N = m.N, P = m.P, G = args.G, C = args.C, S = args.S;
    fill_trig<T>(s_trig, P);
    __syncthreads();
    const int tid = threadIdx.x, grp = tid >> args.logG, g = tid & (G - 1), lane = tid & 31;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    T* qs = s_trig + align_up(2 * P, 4) + grp * args.qstride;
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * S; base < args.X;
         base += static_cast<int64_t>(gridDim.x) * S) {
        const int64_t sidx = base + grp;
        if (sidx < args.X) {
            const int src = draw_sample_smem<T>(m, s_trig, qs, sidx, args.offset, args.key0,
                                                args.key1, g, G, C, g * C, gmask);
            if (args.out.src_out && g == 0) args.out.src_out[sidx] = src;
            const int NP = N * P;
            float* qo = args.out.q_out + sidx * static_cast<int64_t>(NP);
            for (int i = g; i < NP; i += G) qo[i] = static_cast<float>(qs[i]);
        }
        __syncwarp();
    }
}

// host-side launcher, instantiated per surface count in pbr_fused_a*.cu
template <int A>
int launch_fused(int K, int qmode, int precision, const FusedArgs& args, cudaStream_t stream);

}  // namespace pbr
