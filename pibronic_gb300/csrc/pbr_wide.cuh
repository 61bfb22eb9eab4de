// pbr_wide.cuh -- the block evaluation for 9 to 16 surfaces (rows padded to AP = 12 or 16), FP32,
// on the bead coordinates q [X][N][P] and the potential V [X * P][ld] that the sampler and the
// tensor-core potential GEMM wrote for the chunk (both L2-resident).
//
// One CTA of kWideThreads threads evaluates one sample at a time; G teams of kWideTeam threads
// own contiguous chunks of C beads (thread r of a team owns row r of the AP x AP matrices).  The
// beads are taken in windows of W per team:
//
//   B1  two threads per bead (half of the surfaces each): the O-matrix exponents of rho and of the
//       coupled model (beta series of order K), ln S12, the scaled O series and rho log terms,
//       written to a per-bead record in shared memory.
//   B2  per team, bead by bead: M_p = exp(-tau V_p) by scaling and squaring (V shifted by its mean
//       eigenvalue, scaled until ||B||_inf <= 1/2, Taylor degree 8 by Horner, squared back), then
//       N(h) <- N(h) M_p diag(O_p(h)) with the series update done in place (descending order).
//   C   chunk products combined in bead order through shared memory (log2 G levels).
//   D   traces, rho, g(beta +- db) in FP64, as in the row-team form.
//
// Padded rows and columns (A < r < AP) carry zero O entries, so they never reach the trace.
// The reference diagonalises V with numpy.linalg.eigh and exponentiates the eigenvalues
// (pimc.py:1139-1174, 1197-1205); for symmetric V the scaling-and-squaring exponential is the same
// matrix, computed with matrix products only.
#pragma once

#include "pbr_team.cuh"

namespace pbr {

constexpr int kWideThreads = 256;
constexpr int kWideTeam = 16;
constexpr int kWideTeams = kWideThreads / kWideTeam;
constexpr int kWideTaylor = 8;
constexpr int kWideMaxSquarings = 40;

struct WideArgs {
    pbr_model m;
    const float* q;      // [X][N][P]
    const float* vq;     // [X * P][vq_ld], column pair_index(b, c)
    int vq_ld;
    int64_t X;
    pbr_outputs out;
    int G;               // teams per sample
    int C;               // beads per team
    int W;               // beads per team per window
};

__host__ __device__ constexpr int wide_kp(int K) { return (K + 1 + 3) / 4 * 4; }
__host__ __device__ constexpr int wide_mr(int AP, int K) { return 2 * wide_kp(K) + 2 * AP + 4; }
// record: [O series (K+1) x AP][rho log terms AP][ln S12] padded to 4
__host__ __device__ constexpr int wide_rl(int AP, int K) { return ((K + 1) * AP + AP + 1 + 3) / 4 * 4; }

// shared memory (floats): tables | per window: bead records, matrix-exponential buffers and the
// window's V rows (prefetched with cp.async) -- reused by the chunk-combine slots afterwards
struct WidePlan {
    int c, rc, tab, rec, xb, vwin, comb, lsum, total_bytes;
    __host__ __device__ WidePlan(int AP, int K, int N, int G, int W, int ld) {
        int o = 0;
        auto take = [&](int n) { int r = o; o = (o + n + 3) / 4 * 4; return r; };
        c = take((K + 1) * AP);
        rc = take(AP);
        tab = take(N * wide_mr(AP, K));
        const int recs = G * W * wide_rl(AP, K) + kWideTeams * 2 * AP * AP + G * W * ld;
        const int combs = G * ((K + 1) * AP * AP + 4);
        rec = take(recs > combs ? recs : combs);
        xb = rec + G * W * wide_rl(AP, K);
        vwin = xb + kWideTeams * 2 * AP * AP;
        comb = rec;
        lsum = take(G * (AP + 2) * 2);                         // doubles
        total_bytes = o * 4;
    }
};

template <int AP, int K>
__device__ void wide_load_tables(const pbr_model& m, float* sm, const WidePlan& plan) {
    constexpr int KP = wide_kp(K), MR = wide_mr(AP, K);
    const int A = m.A, N = m.N, nfill = m.n_fill_rho;
    float* s_c = sm + plan.c;
    float* s_rc = sm + plan.rc;
    float* s_tab = sm + plan.tab;
    const float* g_cs = static_cast<const float*>(m.vib_cs);
    const float* g_th = static_cast<const float*>(m.vib_th);
    const float* g_c = static_cast<const float*>(m.vib_c);
    const float* g_d = static_cast<const float*>(m.vib_d);
    const float* g_rcs = static_cast<const float*>(m.rho_cs);
    const float* g_rth = static_cast<const float*>(m.rho_th);
    const float* g_rc = static_cast<const float*>(m.rho_c);
    const float* g_rd = static_cast<const float*>(m.rho_d);
    for (int i = threadIdx.x; i < (K + 1) * AP; i += kWideThreads) {
        const int k = i / AP, a = i - k * AP;
        s_c[i] = (a < A) ? g_c[k * A + a] : 0.f;
    }
    for (int i = threadIdx.x; i < AP; i += kWideThreads) s_rc[i] = (i < nfill) ? g_rc[i] : 0.f;
    for (int i = threadIdx.x; i < N * MR; i += kWideThreads) {
        const int j = i / MR, o = i - j * MR;
        float v = 0.f;
        if (o < KP) { if (o <= K) v = g_cs[o * N + j]; }
        else if (o < 2 * KP) { if (o - KP <= K) v = g_th[(o - KP) * N + j]; }
        else if (o < 2 * KP + AP) { const int a = o - 2 * KP; if (a < A) v = g_d[a * N + j]; }
        else if (o < 2 * KP + 2 * AP) { const int a = o - 2 * KP - AP; if (a < nfill) v = g_rd[a * N + j]; }
        else if (o == 2 * KP + 2 * AP) v = g_rcs[j];
        else if (o == 2 * KP + 2 * AP + 1) v = g_rth[j];
        s_tab[i] = v;
    }
}

// team-wide reductions over the kWideTeam threads of a team (aligned within a warp)
__device__ __forceinline__ float team_max(float v, unsigned mask) {
#pragma unroll
    for (int o = kWideTeam / 2; o >= 1; o >>= 1) v = fmaxf(v, __shfl_xor_sync(mask, v, o, kWideTeam));
    return v;
}
__device__ __forceinline__ float team_sum(float v, unsigned mask) {
#pragma unroll
    for (int o = kWideTeam / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(mask, v, o, kWideTeam);
    return v;
}

// out = x X for the row x of this thread and the AP x AP matrix X in shared memory (broadcast reads)
template <int AP>
__device__ __forceinline__ void row_times(const float (&x)[AP], const float* X, float (&out)[AP]) {
#pragma unroll
    for (int c = 0; c < AP; ++c) out[c] = 0.f;
#pragma unroll
    for (int mm = 0; mm < AP; ++mm) {
        // at most four rows of X in flight: keeps the unrolled loads from crowding the registers
        if ((mm & 3) == 0) asm volatile("" ::: "memory");
        float row[AP];
        ldv(X + mm * AP, row);
#pragma unroll
        for (int c = 0; c < AP; ++c) out[c] = fmaf(x[mm], row[c], out[c]);
    }
}

template <int AP, int K>
__device__ void wide_sample(const WideArgs& args, float* sm, const WidePlan& plan, int64_t x) {
    constexpr int AH = AP / 2;
    constexpr int KP = wide_kp(K), MR = wide_mr(AP, K), RL = wide_rl(AP, K);
    constexpr int OFF_R = (K + 1) * AP, OFF_L = OFF_R + AP;
    constexpr int CL = (K + 1) * AP * AP + 4;
    const pbr_model& m = args.m;
    const int A = m.A, N = m.N, P = m.P, nfill = m.n_fill_rho;
    const int G = args.G, C = args.C, W = args.W;
    const float tau = static_cast<float>(m.tau);
    const float* s_c = sm + plan.c;
    const float* s_rc = sm + plan.rc;
    const float* s_tab = sm + plan.tab;
    float* s_rec = sm + plan.rec;
    double* s_lsum = reinterpret_cast<double*>(sm + plan.lsum);
    const int tid = threadIdx.x, lane = tid & 31;
    const int team = tid / kWideTeam, r = tid % kWideTeam;
    const unsigned tmask = 0xFFFFu << (lane & ~(kWideTeam - 1));
    const bool tact = team < G;
    float* xb0 = sm + plan.xb + team * 2 * AP * AP;
    float* xb1 = xb0 + AP * AP;
    const float* qx = args.q + x * static_cast<int64_t>(N) * P;
    const float* vx = args.vq + x * static_cast<int64_t>(P) * args.vq_ld;

    float nrow[K + 1][AP];
    int nexp = 0;
    LogSum<float> lr, ls;
    const int pb = team * C, pe = min(P, pb + C);
#pragma unroll
    for (int k = 0; k <= K; ++k)
#pragma unroll
        for (int c = 0; c < AP; ++c) nrow[k][c] = 0.f;
    const int nwin = (C + W - 1) / W;

    float* s_vwin = sm + plan.vwin;
    const int ld = args.vq_ld;
    for (int w = 0; w < nwin; ++w) {
        // the window's V rows, copied asynchronously while the records are computed
        for (int idx = tid; idx < G * W * (ld / 4); idx += kWideThreads) {
            const int sl = idx / (ld / 4), ch = idx - sl * (ld / 4);
            const int g = sl / W, lp = w * W + (sl - g * W);
            const int p = g * C + lp;
            if (lp < C && p < P)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                             ::"r"(static_cast<uint32_t>(__cvta_generic_to_shared(s_vwin + sl * ld + 4 * ch))),
                               "l"(vx + static_cast<int64_t>(p) * ld + 4 * ch) : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        // ================================ phase B1: bead records ===============================
        for (int sl0 = 0; sl0 < G * W; sl0 += kWideThreads / 2) {     // uniform trip count
            const int sl = sl0 + (tid >> 1);
            const int g = sl / W, i = sl - g * W;
            const int lp = w * W + i;
            const int p = g * C + lp;
            const bool valid = sl < G * W && lp < C && p < P;
            const int half = tid & 1;
            float phv[K + 1][AH], phr[AH];
#pragma unroll
            for (int k = 0; k <= K; ++k)
#pragma unroll
                for (int a = 0; a < AH; ++a) phv[k][a] = s_c[k * AP + half * AH + a];
#pragma unroll
            for (int a = 0; a < AH; ++a) phr[a] = s_rc[half * AH + a];
            float dsum[K + 1];
#pragma unroll
            for (int k = 0; k <= K; ++k) dsum[k] = 0.f;
            float rdsum = 0.f;
            if (valid) {
                const int pn = (p + 1 == P) ? 0 : p + 1;
#pragma unroll 2
                for (int j = 0; j < N; ++j) {
                    const float* rec = s_tab + j * MR;
                    float cs[KP], th[KP], dv[AH], rdv[AH], rx[4];
                    ldv(rec, cs);
                    ldv(rec + KP, th);
#pragma unroll
                    for (int a = 0; a < AH; ++a) {
                        dv[a] = rec[2 * KP + half * AH + a];
                        rdv[a] = rec[2 * KP + AP + half * AH + a];
                    }
                    ldv(rec + 2 * KP + 2 * AP, rx);
                    const float qa = __ldg(qx + j * P + p), qb = __ldg(qx + j * P + pn);
                    const float dq = qa - qb, dq2 = dq * dq;
#pragma unroll
                    for (int k = 0; k <= K; ++k) dsum[k] = fmaf(cs[k], dq2, dsum[k]);
                    rdsum = fmaf(rx[0], dq2, rdsum);
#pragma unroll
                    for (int a = 0; a < AH; ++a) {
                        const float ua = qa - dv[a], ub = qb - dv[a];
                        const float sq = fmaf(ua, ua, ub * ub);
#pragma unroll
                        for (int k = 0; k <= K; ++k) phv[k][a] = fmaf(-th[k], sq, phv[k][a]);
                        const float ra = qa - rdv[a], rb = qb - rdv[a];
                        phr[a] = fmaf(-rx[1], fmaf(ra, ra, rb * rb), phr[a]);
                    }
                }
            }
            float lmax = -INFINITY;
#pragma unroll
            for (int a = 0; a < AH; ++a) {
                const int ag = half * AH + a;
#pragma unroll
                for (int k = 0; k <= K; ++k) phv[k][a] -= dsum[k];
                phr[a] -= rdsum;
                if (ag < A) lmax = fmaxf(lmax, phv[0][a]);
                if (ag < nfill) lmax = fmaxf(lmax, phr[a]);
            }
            lmax = fmaxf(lmax, __shfl_xor_sync(0xffffffffu, lmax, 1));
            if (valid) {
                float* ro = s_rec + sl * RL;
                if (half == 0) ro[OFF_L] = lmax;
#pragma unroll
                for (int a = 0; a < AH; ++a) {
                    const int ag = half * AH + a;
                    ro[OFF_R + ag] = (ag < nfill) ? phr[a] - lmax : 0.f;
                    float ek[K + 1];
                    ek[0] = 1.f;
#pragma unroll
                    for (int k = 1; k <= K; ++k) {
                        float acc = 0.f;
#pragma unroll
                        for (int i2 = 1; i2 <= k; ++i2) acc = fmaf(float(i2) * phv[i2][a], ek[k - i2], acc);
                        ek[k] = acc * (1.f / float(k));
                    }
                    const float e0 = (ag < A) ? dev_exp<float>(phv[0][a] - lmax) : 0.f;
#pragma unroll
                    for (int k = 0; k <= K; ++k) ro[k * AP + ag] = e0 * ek[k];
                }
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();

        // ================================ phase B2: exp(-tau V), ring product ==================
        if (tact) {
            for (int i = 0; i < W; ++i) {
                const int lp = w * W + i;
                const int p = pb + lp;
                if (lp >= C || p >= pe) break;                 // team-uniform
                // V row r (symmetric, packed pairs), padded with zeros
                float b[AP];
                const float* vr = s_vwin + (team * W + i) * ld;
                float dg = 0.f;
#pragma unroll
                for (int c = 0; c < AP; ++c) {
                    const int hi = r > c ? r : c, lo = r > c ? c : r;
                    b[c] = (r < A && c < A) ? vr[hi * (hi + 1) / 2 + lo] : 0.f;
                    if (c == r) dg = b[c];
                }
                const float vmean = team_sum(dg, tmask) / float(A);
                float rs = 0.f;
#pragma unroll
                for (int c = 0; c < AP; ++c) {
                    b[c] = (r < A && c < A) ? -tau * (b[c] - (c == r ? vmean : 0.f)) : 0.f;
                    rs += fabsf(b[c]);
                }
                float nrm = team_max(rs, tmask);
                int s = 0;
                while (nrm > 0.5f && s < kWideMaxSquarings) { nrm *= 0.5f; ++s; }
                const float sc = ldexpf(1.f, -s);
#pragma unroll
                for (int c = 0; c < AP; ++c) b[c] *= sc;
                // Taylor polynomial of degree 8, Paterson-Stockmeyer: with C_i = c_3i I + c_3i+1 B +
                // c_3i+2 B^2 (c_k = 1/k!), exp(B) ~ C_0 + B^3 (C_1 + B^3 C_2): four matrix products
                float* x0 = xb0;
                float* x1 = xb1;
                if (r < AP) stv(x0 + r * AP, b);
                __syncwarp(tmask);
                float b2[AP], xr[AP];
                row_times<AP>(b, x0, b2);
                row_times<AP>(b2, x0, xr);                      // row of B^3
                if (r < AP) stv(x1 + r * AP, xr);
                __syncwarp(tmask);
                constexpr float c3 = 1.f / 6.f, c4 = 1.f / 24.f, c5 = 1.f / 120.f, c6 = 1.f / 720.f,
                                c7 = 1.f / 5040.f, c8 = 1.f / 40320.f;
                {
                    float t[AP];
#pragma unroll
                    for (int c = 0; c < AP; ++c) t[c] = (c == r ? c6 : 0.f) + c7 * b[c] + c8 * b2[c];
                    row_times<AP>(t, x1, xr);                   // C_2 B^3
#pragma unroll
                    for (int c = 0; c < AP; ++c) t[c] = (c == r ? c3 : 0.f) + c4 * b[c] + c5 * b2[c] + xr[c];
                    row_times<AP>(t, x1, xr);                   // (C_1 + C_2 B^3) B^3
#pragma unroll
                    for (int c = 0; c < AP; ++c) xr[c] += (c == r ? 1.f : 0.f) + b[c] + 0.5f * b2[c];
                }
                // squarings; x0 / x1 alternate (every row of the buffer read is complete before
                // it is replaced: a warp barrier separates each write from the reads before it)
                float* cur = x0;
                float* nxt = x1;
                for (int sq = 0; sq < s; ++sq) {
                    if (r < AP) stv(cur + r * AP, xr);
                    __syncwarp(tmask);
                    float t[AP];
                    row_times<AP>(xr, cur, t);
#pragma unroll
                    for (int c = 0; c < AP; ++c) xr[c] = t[c];
                    float* tmp = cur; cur = nxt; nxt = tmp;
                }
                // M = 2^(t - n2) X with t = -tau vmean log2(e); the power of two goes to nexp
                const float tl = -tau * vmean * 1.4426950408889634f;
                const float n2 = floorf(tl);
                const float f = exp2f(tl - n2);
                nexp += static_cast<int>(n2);
#pragma unroll
                for (int c = 0; c < AP; ++c) xr[c] *= f;
                if (r < AP) stv(cur + r * AP, xr);
                __syncwarp(tmask);
                const float* M = cur;
                const float* rc_ = s_rec + (team * W + i) * RL;
                if (r == 0) ls.add(rc_[OFF_L]);
                if (r < nfill) lr.add(rc_[OFF_R + (r < AP ? r : 0)]);
                if (p == pb) {
#pragma unroll
                    for (int k = 0; k <= K; ++k) {
                        float os[AP];
                        ldv(rc_ + k * AP, os);
#pragma unroll
                        for (int c = 0; c < AP; ++c) nrow[k][c] = (r < A) ? xr[c] * os[c] : 0.f;
                    }
                } else {
#pragma unroll
                    for (int ii = K; ii >= 0; --ii) {
                        // re-read M per series term rather than holding all of it in registers
                        asm volatile("" ::: "memory");
                        float y[AP];
                        row_times<AP>(nrow[ii], M, y);
                        float os[AP];
                        ldv(rc_, os);
#pragma unroll
                        for (int c = 0; c < AP; ++c) nrow[ii][c] = y[c] * os[c];
#pragma unroll
                        for (int k = ii + 1; k <= K; ++k) {
                            ldv(rc_ + (k - ii) * AP, os);
#pragma unroll
                            for (int c = 0; c < AP; ++c) nrow[k][c] = fmaf(y[c], os[c], nrow[k][c]);
                        }
                    }
                }
                if (((p - pb) & 1) == 1 || p + 1 == pe) {
                    float mx = 0.f;
#pragma unroll
                    for (int c = 0; c < AP; ++c) mx = fmaxf(mx, fabsf(nrow[0][c]));
                    mx = team_max(mx, tmask);
                    if (mx > 0.f && isfinite(mx)) {
                        int e2;
                        frexpf(mx, &e2);
                        const float scl = ldexpf(1.f, -e2);
                        nexp += e2;
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < AP; ++c) nrow[k][c] *= scl;
                    }
                }
                __syncwarp(tmask);            // M and the record are read before the next bead
            }
        }
        __syncthreads();
    }
    if (tact && pb >= pe) {
#pragma unroll
        for (int k = 0; k <= K; ++k)
#pragma unroll
            for (int c = 0; c < AP; ++c) nrow[k][c] = (k == 0 && c == r && r < A) ? 1.f : 0.f;
    }

    // ================================ phase C: combine chunks ==================================
    // Each team's series rows go to its slot; a receiving team multiplies its slot by the partner's
    // in place (descending series order: z_k = sum_{i <= k} own_i Y_{k-i} only reads own_i, i <= k).
    float* comb = s_rec + plan.comb - plan.rec;
    int* cexp = reinterpret_cast<int*>(s_lsum + G * (AP + 1));
    double lr_d = 0.0, ls_d = 0.0;
    float* own = comb + team * CL;
    if (tact) {
        lr_d = lr.value();
        ls_d = ls.value();
        if (r < AP)
#pragma unroll
            for (int k = 0; k <= K; ++k) stv(own + (k * AP + r) * AP, nrow[k]);
        if (r < AP) s_lsum[team * (AP + 1) + r] = lr_d;
        if (r == 0) { s_lsum[team * (AP + 1) + AP] = ls_d; cexp[team] = nexp; }
    }
    __syncthreads();
    for (int st = 1; st < G; st <<= 1) {
        const bool recv = tact && (team % (2 * st)) == 0 && team + st < G;
        if (recv) {
            const int ps = team + st;
            const float* Y = comb + ps * CL;
            float mx = 0.f;
#pragma unroll 1
            for (int k = K; k >= 0; --k) {
                float z[AP];
#pragma unroll
                for (int c = 0; c < AP; ++c) z[c] = 0.f;
                if (r < AP) {
#pragma unroll 1
                    for (int i = 0; i <= k; ++i) {
                        float x[AP], t[AP];
                        ldv(own + (i * AP + r) * AP, x);
                        row_times<AP>(x, Y + (k - i) * AP * AP, t);
#pragma unroll
                        for (int c = 0; c < AP; ++c) z[c] += t[c];
                    }
                }
                __syncwarp(tmask);                    // every row of own_k is read before it is replaced
                if (r < AP) stv(own + (k * AP + r) * AP, z);
                if (k == 0)
#pragma unroll
                    for (int c = 0; c < AP; ++c) mx = fmaxf(mx, fabsf(z[c]));
            }
            if (r < AP) lr_d += s_lsum[ps * (AP + 1) + r];
            if (r == 0) ls_d += s_lsum[ps * (AP + 1) + AP];
            nexp += cexp[ps];
            mx = team_max(mx, tmask);
            if (mx > 0.f && isfinite(mx)) {
                int e2;
                frexpf(mx, &e2);
                const float scl = ldexpf(1.f, -e2);
                nexp += e2;
                if (r < AP)
                    for (int k = 0; k <= K; ++k) {
                        float z[AP];
                        ldv(own + (k * AP + r) * AP, z);
#pragma unroll
                        for (int c = 0; c < AP; ++c) z[c] *= scl;
                        stv(own + (k * AP + r) * AP, z);
                    }
            }
            if (r < AP) s_lsum[team * (AP + 1) + r] = lr_d;
            if (r == 0) { s_lsum[team * (AP + 1) + AP] = ls_d; cexp[team] = nexp; }
        }
        __syncthreads();
    }

    // ================================ phase D: outputs =========================================
    if (team == 0) {
        double coef[K + 1];
#pragma unroll
        for (int k = 0; k <= K; ++k) {
            // the trace summed in FP32 across the team (the entries carry FP32 rounding already)
            float d = (r < A) ? own[(k * AP + r) * AP + r] : 0.f;
#pragma unroll
            for (int o = kWideTeam / 2; o >= 1; o >>= 1) d += __shfl_xor_sync(tmask, d, o, kWideTeam);
            coef[k] = scale_pow2(static_cast<double>(d), nexp);
        }
        double rho = (r < nfill) ? exp_out<float>(lr_d) : 0.0;
#pragma unroll
        for (int o = kWideTeam / 2; o >= 1; o >>= 1) rho += __shfl_xor_sync(tmask, rho, o, kWideTeam);
        if (r == 0) {
            const pbr_outputs& o = args.out;
            o.s_rho[x] = rho;
            o.s_g[x] = coef[0];
            bool bad = !isfinite(rho) || !isfinite(coef[0]);
            if (K > 0) {
                const double db = m.delta_beta;
                double gp = 0.0, gm = 0.0;
#pragma unroll
                for (int k = K; k >= 0; --k) { gp = gp * db + coef[k]; gm = gm * (-db) + coef[k]; }
                if (o.s_gp) o.s_gp[x] = gp;
                if (o.s_gm) o.s_gm[x] = gm;
                bad = bad || !isfinite(gp) || !isfinite(gm);
            }
            if (o.g_coef) {
#pragma unroll
                for (int k = 0; k <= K; ++k) o.g_coef[x * (K + 1) + k] = coef[k];
            }
            if (o.log_scale) o.log_scale[x] = ls_d + static_cast<double>(P) * m.log_c0;
            if (bad) flag_status(o.status, PBR_ERR_NONFINITE);
        }
    }
    __syncthreads();
}

// MB: blocks per SM the registers are sized for (two at AP = 12: 128 registers; one at AP = 16)
template <int AP> constexpr int wide_min_blocks() { return AP <= 12 ? 2 : 1; }

template <int AP, int K, int MB = wide_min_blocks<AP>()>
__global__ void __launch_bounds__(kWideThreads, MB) pimc_wide_kernel(const WideArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sm = reinterpret_cast<float*>(smem_raw);
    const WidePlan plan(AP, K, args.m.N, args.G, args.W, args.vq_ld);
    wide_load_tables<AP, K>(args.m, sm, plan);
    __syncthreads();
    for (int64_t x = blockIdx.x; x < args.X; x += gridDim.x) wide_sample<AP, K>(args, sm, plan, x);
}

// Host side (one instantiation per padded width AP and series order K).  A block evaluates one
// sample at a time, so the caller sizes its chunks in whole waves of wide_resident() samples.
template <int AP, int K, int MB>
int wide_blocks_resident(const WideArgs& args, int* resident) {
    const WidePlan plan(AP, K, args.m.N, args.G, args.W, args.vq_ld);
    auto kern = pimc_wide_kernel<AP, K, MB>;
    if (plan.total_bytes > 227 * 1024) return PBR_ERR_UNSUPPORTED;
    static int configured = 0;
    if (plan.total_bytes > 48 * 1024 && plan.total_bytes > configured) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, plan.total_bytes) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        configured = plan.total_bytes;
    }
    int dev = 0, sms = 0, occ = 0;
    PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
    PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kWideThreads, plan.total_bytes));
    if (occ < 1) return PBR_ERR_UNSUPPORTED;
    *resident = occ * sms;
    return PBR_OK;
}

template <int AP, int K, int MB>
int launch_wide_one(const WideArgs& args, cudaStream_t stream) {
    int resident = 0;
    const int rc = wide_blocks_resident<AP, K, MB>(args, &resident);
    if (rc != PBR_OK) return rc;
    const int64_t grid = args.X < resident ? args.X : resident;
    if (grid <= 0) return PBR_OK;
    const WidePlan plan(AP, K, args.m.N, args.G, args.W, args.vq_ld);
    pimc_wide_kernel<AP, K, MB><<<static_cast<int>(grid), kWideThreads, plan.total_bytes, stream>>>(args);
    return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
}

template <int AP>
int launch_wide(int K, const WideArgs& args, cudaStream_t stream) {
    constexpr int MB = wide_min_blocks<AP>();
    return K == 0 ? launch_wide_one<AP, 0, MB>(args, stream) : launch_wide_one<AP, 4, MB>(args, stream);
}

// blocks launch_wide keeps resident (0 when it cannot run)
template <int AP>
int wide_resident(int K, const WideArgs& args) {
    constexpr int MB = wide_min_blocks<AP>();
    int resident = 0;
    const int rc = K == 0 ? wide_blocks_resident<AP, 0, MB>(args, &resident)
                          : wide_blocks_resident<AP, 4, MB>(args, &resident);
    return rc == PBR_OK ? resident : 0;
}

}  // namespace pbr
