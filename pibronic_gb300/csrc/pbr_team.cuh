// pbr_team.cuh -- the fused PIMC block evaluation, bead-parallel / row-team form.
//
// One CTA of kTeamThreads threads evaluates S samples per tile in four block-synchronised phases:
//
//   A   q[j][p] of the tile's samples into shared memory (device sampler, block-cooperative:
//       sources, Philox normals, real-Fourier ring transform; or the caller's q).
//   B1  one thread per (sample, bead): O-matrix exponents of rho and the coupled model (beta
//       series of order K), ln S12, the scaled O series, V(q_p), Jacobi, M_p = U exp(-tau lambda) U^T;
//       written to a per-bead record in shared memory.
//   B2  a team of TA = pow2ceil(A) threads per bead chunk, thread r owning row r of the series
//       matrices N_k: N(h) <- N(h) M_p diag(O_p(h)) over the chunk, power-of-two renormalised.
//   C   chunk products combined in bead order through shared memory (log2 G levels).
//   D   traces, rho, g(beta +- db) in FP64; one team per sample writes the outputs.
//
// Registers per thread stay near the B1 working set (V, Jacobi, one bead's series), so far more
// warps are resident than in the register-resident chunk form, and A up to 8 fits.
#pragma once

#include "pbr_fused.cuh"

namespace pbr {

constexpr int kTeamThreads = 256;
// largest surface count whose exp(-tau V) is formed by scaling and squaring in one thread's
// registers (FP32); beyond it the per-thread Jacobi of the FP64 form is used
constexpr int kTeamExpmMaxA = 8;

struct TeamArgs {
    pbr_model m;
    const void* q_in;
    int64_t X;
    pbr_outputs out;
    uint32_t key0, key1;
    uint64_t offset;
    int S;          // samples per tile
    int G;          // teams (bead chunks) per sample, a power of two
    int C;          // beads per team
    int rs;         // q row stride (skewed layout, qidx)
    int qstride;    // q elements per sample
    int rl;         // bead record length
    const float* vq;  // kQ32V: V(q) (energies, linear, quadratic), row (sample * P + bead), A(A+1)/2 used columns
    int vq_ld;        // kQ32V: floats per row of vq
    int tcq;          // 1: B1's quadratic part of V on the tensor cores (its tables, its instantiation)
};

__host__ __device__ inline int pow2_ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// bead record: [M: A*A][O series: (K+1)*A][ln S12][M exponent][rho log terms: A].  From 6
// surfaces on, M and the O series are each padded to a multiple of 4 so that both sit at 16-byte
// offsets with whole float4 lengths (128-bit loads in the row teams; no change in length at 6
// and 8 surfaces).  The record length is an odd multiple of 4 floats: in B1 the 32 threads of a
// warp write 32 consecutive records, so a length that is a multiple of 32 (the unpadded record at
// 3 surfaces, 32; at 7, 96) puts every store of the warp in one shared-memory bank, 32-way
// conflicts, where an odd multiple of 4 gives 4-way (the 7-surface batch group ran 1.4x faster
// for going from 96 to 100).  Below 6 surfaces M and O stay unpadded: at 5 the padding would grow
// the record by 13 % and move models out of the two-block build.
__host__ __device__ constexpr int record_pad(int n, int A) { return A >= 6 ? (n + 3) / 4 * 4 : n; }
__host__ __device__ constexpr int record_off_o(int A) { return record_pad(A * A, A); }
__host__ __device__ constexpr int record_off_l(int A, int K) { return record_off_o(A) + record_pad((K + 1) * A, A); }
__host__ __device__ inline int record_len(int A, int K) {
    const int n = align_up(record_off_l(A, K) + 2 + A, 4);
    return (n & 4) ? n : n + 4;
}

// Combine-slot length: the (K+1) A x A series matrices of a chunk product plus 4, padded so that
// the slots of the four teams of a warp, each writing its A rows A floats apart, fall in distinct
// banks (the pad per surface count that gives the fewest store wavefronts for K = 4 and K = 0;
// unpadded, the 7-surface slots of 249 floats put two teams in the same banks: 4x the wavefronts).
__host__ __device__ inline int comb_len(int A, int K) {
    constexpr int pad4[9] = {0, 0, 1, 3, 1, 0, 3, 15, 1};
    constexpr int pad0[9] = {0, 0, 1, 7, 1, 0, 3, 3, 1};
    const int a = A < 0 ? 0 : (A > 8 ? 8 : A);
    return (K + 1) * A * A + 4 + (K > 0 ? pad4[a] : pad0[a]);
}

struct TeamPlan {
    int c, e, qq, rc, rec, src, q, qlo, beads, lsums, total_bytes;
    int alt;          // second buffer of combine slots (the split combine), or -1: none fits
    bool stage_ring;  // the ring factor fits the bead-record region (phase A copies it there)
    int tcq_k;        // k-steps of B1's tensor-core quadratic (0: the FP32 pair loop)
    __host__ __device__ TeamPlan() : c(0), e(0), qq(0), rc(0), rec(0), src(0), q(0), qlo(0), beads(0),
                                     lsums(0), total_bytes(0), alt(-1), stage_ring(false), tcq_k(0) {}
    __host__ __device__ TeamPlan(int A, int K, int qm, int esz, int N, int P, int S, int G, int qstride,
                                 int rl, int tcq = 0) {
        const int A2P = align_up(npair(A), 4);
        int o = 0;
        auto take = [&](int n) { int r = o; o = align_up(o + n, 4); return r; };
        tcq_k = (tcq && esz == 4 && qm != kQ32V && N >= kTcqMinN && qstride - 1 < 65536) ? tcq_ksteps(N) : 0;
        c = take((K + 1) * A); e = take(A2P);
        qq = take(qm == kQ32V ? 0 : (tcq_k ? tcq_words(N, A) : npair(N) * A2P)); rc = take(A);
        rec = take(N * rec_len(A, K));
        src = take(S);                                             // ints stored in the slot
        q = take(S * qstride);
        qlo = take((qm == kQ64 && esz == 4) ? S * qstride : 0);
        const int comb = S * G * comb_len(A, K);
        int nb = S * P * rl;
        nb = nb > comb ? nb : comb;
        beads = take(nb);
        // the split combine's second slot buffer: the rest of the bead-record region, else the q
        // tile (both are free once B1 is done)
        alt = (nb >= 2 * comb) ? beads + comb : (S * qstride >= comb ? q : -1);
        stage_ring = 3 * N * P <= nb && (beads * esz) % 16 == 0;
        lsums = take((S * G * (A + 2) * 8 + esz - 1) / esz);      // 8-byte log sums + exponent slot
        total_bytes = o * esz;
    }
};

// Copy one model's tables into the CTA's shared memory (layout TeamPlan; kTcq: the tensor-core
// quadratic's tables in place of the packed coupling table, its mode offsets in rows of rs).
template <int A, int K, int QM, typename T, bool kTcq = false>
__device__ void team_load_tables(const pbr_model& m, int rs, T* sm, const TeamPlan& plan) {
    constexpr int A2 = npair(A);
    constexpr int A2P = (A2 + 3) / 4 * 4;
    constexpr int KP = (K + 1 + 3) / 4 * 4;
    constexpr int AP = (A + 3) / 4 * 4;
    constexpr int MR = 2 * KP + 2 * AP + 4 + A2P;
    constexpr int NT = kTeamThreads;
    const int N = m.N, nfill = m.n_fill_rho;
    const int tid = threadIdx.x;
    T* s_c = sm + plan.c;    T* s_e = sm + plan.e;    T* s_qq = sm + plan.qq;
    T* s_rc = sm + plan.rc;  T* s_rec = sm + plan.rec;
    {
        const T* g_cs = static_cast<const T*>(m.vib_cs);  const T* g_th = static_cast<const T*>(m.vib_th);
        const T* g_c = static_cast<const T*>(m.vib_c);    const T* g_d = static_cast<const T*>(m.vib_d);
        const T* g_e = static_cast<const T*>(m.vib_e);    const T* g_l = static_cast<const T*>(m.vib_l);
        const T* g_qq = static_cast<const T*>(m.vib_qq);
        const T* g_rcs = static_cast<const T*>(m.rho_cs); const T* g_rth = static_cast<const T*>(m.rho_th);
        const T* g_rc = static_cast<const T*>(m.rho_c);   const T* g_rd = static_cast<const T*>(m.rho_d);
        for (int i = tid; i < (K + 1) * A; i += NT) s_c[i] = g_c[i];
        for (int i = tid; i < A2P; i += NT) s_e[i] = (i < A2) ? g_e[i] : T(0);
        if constexpr (kTcq) {
            tcq_tables<A>(reinterpret_cast<const float*>(g_qq), N, rs, plan.tcq_k,
                          reinterpret_cast<uint32_t*>(s_qq));
        } else {
            const int N2 = (QM == kQ32V) ? 0 : npair(N);
            for (int i = tid; i < N2 * A2P; i += NT) {
                const int row = i / A2P, col = i - row * A2P;
                s_qq[i] = (col < A2) ? g_qq[row * A2 + col] : T(0);
            }
        }
        for (int i = tid; i < A; i += NT) s_rc[i] = (i < nfill) ? g_rc[i] : T(0);
        for (int i = tid; i < N * MR; i += NT) {
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
}

// One tile of S samples starting at global sample `base` (phases A, B1, B2, C, D); ends with a
// block barrier, so the caller may reload the tables afterwards.  MB is the blocks per SM the
// build targets; the two-block build (128 registers) uses the forms that need fewer registers:
// the receiver combine, a two-step prefetch in the chains and, at 5 surfaces, a B2 that streams
// the bead matrices column by column (at 6 surfaces that form measured slower than its spills).
template <int A, int K, int QM, typename T, int MB = 1, bool kTcq = false>
__device__ void team_tile(const TeamArgs& args, T* sm, const TeamPlan& plan, int64_t base) {
    constexpr int A2 = npair(A);
    constexpr int A2P = (A2 + 3) / 4 * 4;
    constexpr int KP = (K + 1 + 3) / 4 * 4;
    constexpr int AP = (A + 3) / 4 * 4;
    constexpr int MR = 2 * KP + 2 * AP + 4 + A2P;
    constexpr int TA = (A <= 1) ? 1 : (A <= 2) ? 2 : (A <= 4) ? 4 : 8;
    constexpr int OFF_O = record_off_o(A), OFF_L = record_off_l(A, K), OFF_N = OFF_L + 1, OFF_R = OFF_L + 2;
    // the O block takes 128-bit stores and loads only at a 16-byte offset
    static_assert(OFF_O % 4 == 0 || (OFF_L - OFF_O) % 4 != 0, "O block length a multiple of 4 at an unaligned offset");
    constexpr bool kLo = (QM == kQ64) && (sizeof(T) == 4);
    constexpr int NT = kTeamThreads;
    constexpr bool kTwoBlock = MB > 1;
    constexpr bool kLeanB2 = kTwoBlock && A == 5;

    const pbr_model& m = args.m;
    const int N = m.N, P = m.P, nfill = m.n_fill_rho, rs = args.rs;
    const int S = args.S, G = args.G, C = args.C, RL = args.rl;
    T* s_c = sm + plan.c;    T* s_e = sm + plan.e;    T* s_qq = sm + plan.qq;
    T* s_rc = sm + plan.rc;  T* s_rec = sm + plan.rec;
    int* s_src = reinterpret_cast<int*>(sm + plan.src);
    T* s_q = sm + plan.q;
    T* s_ql = kLo ? sm + plan.qlo : nullptr;
    T* s_beads = sm + plan.beads;
    // per combine slot: the team's compensated log sums (rho terms, ln S12), 8 bytes each
    LogSum<T>* s_lsum = reinterpret_cast<LogSum<T>*>(sm + plan.lsums);
    const int tid = threadIdx.x;


    const T tau_l2 = T(m.tau * 1.4426950408889634);   // tau * log2(e)
    const int NP = N * P;
    // B2 / C / D thread roles
    const int team = tid / TA, r = tid % TA;
    const int ts = team / G, tc = team % G;               // sample slot and chunk of this team
    const bool team_ok = team < S * G;
    const int lane = tid & 31;
    const unsigned tmask = (TA == 32) ? 0xffffffffu : (((1u << TA) - 1u) << (lane & ~(TA - 1)));
    const int CL = comb_len(A, K);                         // combine slot length

    {
        const int nvalid = static_cast<int>(min(static_cast<int64_t>(S), args.X - base));

        // ================================ phase A ==============================================
        if (QM == kSample) {
            // The ring factor [3][P][N] is copied asynchronously into the bead-record region (free
            // until B1) when it fits: the chains below then read shared memory, not L2.
            const T* tab = static_cast<const T*>(m.ring_chol);
            const bool stage = plan.stage_ring && (reinterpret_cast<uintptr_t>(tab) & 15) == 0;
            if (stage) {
                const int nbytes = 3 * N * P * static_cast<int>(sizeof(T));
                const char* gsrc = reinterpret_cast<const char*>(tab);
                const uint32_t sdst = static_cast<uint32_t>(__cvta_generic_to_shared(s_beads));
                for (int o = 16 * tid; o + 16 <= nbytes; o += 16 * NT)
                    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" :: "r"(sdst + o), "l"(gsrc + o) : "memory");
                for (int o = (nbytes & ~15) + 4 * tid; o < nbytes; o += 4 * NT)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" :: "r"(sdst + o), "l"(gsrc + o) : "memory");
                asm volatile("cp.async.commit_group;" ::: "memory");
                tab = s_beads;
            }
            for (int s = tid; s < S; s += NT)
                s_src[s] = (s < nvalid) ? draw_source<T>(m, args.offset + static_cast<uint64_t>(base + s),
                                                         args.key0, args.key1) : 0;
            // the tile's normals over all threads, then one back-substitution chain per (sample, mode)
            fill_normals<T>(m, s_q, args.qstride, rs, nvalid, args.offset + static_cast<uint64_t>(base),
                            args.key0, args.key1, tid, NT);
            if (stage) asm volatile("cp.async.wait_all;" ::: "memory");
            __syncthreads();
            for (int it = tid; it < nvalid * N; it += NT) {
                const int s = it / N, j = it - s * N;
                const T dsh = static_cast<const T*>(m.rho_d)[static_cast<int64_t>(s_src[s]) * N + j];
                back_substitute<T, kTwoBlock ? 2 : kBsGroup>(tab, N, P, j, dsh, s_q + s * args.qstride + j * rs);
            }
            __syncthreads();
            if (args.out.q_out) {
                // a warp per (sample, mode) row, lanes over the beads (no per-element division)
                for (int row = tid >> 5; row < nvalid * N; row += NT >> 5) {
                    const int s = row / N, j = row - s * N;
                    float* dst = args.out.q_out + ((base + s) * N + j) * static_cast<int64_t>(P);
                    const T* src = s_q + s * args.qstride + j * rs;
                    for (int p = tid & 31; p < P; p += 32) dst[p] = static_cast<float>(src[p + (p >> 5)]);
                }
            }
            if (args.out.src_out)
                for (int s = tid; s < nvalid; s += NT) args.out.src_out[base + s] = s_src[s];
        } else {
            // the caller's q: a warp per (sample, mode) row, lanes over the beads
            for (int row = tid >> 5; row < nvalid * N; row += NT >> 5) {
                const int s = row / N, j = row - s * N;
                const int64_t src0 = ((base + s) * N + j) * static_cast<int64_t>(P);
                T* dq = s_q + s * args.qstride + j * rs;
                T* dl = kLo ? s_ql + s * args.qstride + j * rs : nullptr;
                for (int p = tid & 31; p < P; p += 32) {
                    const int d = p + (p >> 5);                      // qidx(j, p, rs) - j * rs
                    if (QM == kQ64) {
                        const double v = static_cast<const double*>(args.q_in)[src0 + p];
                        const T hi = T(v);
                        dq[d] = hi;
                        if (kLo) dl[d] = T(v - static_cast<double>(hi));
                    } else {
                        dq[d] = T(static_cast<const float*>(args.q_in)[src0 + p]);
                    }
                }
            }
            __syncthreads();
        }

        // ================================ phase B1: bead records ===============================
        // record it = (sample s, bead p); on = a live record.  With the tensor-core quadratic every
        // thread runs the same number of records (the warp's 32 rows go through the MMAs
        // together); otherwise each thread takes its own records only.
        int it_base = 0;           // first record of the current round (the uniform loop)
        auto record = [&](const int it, const bool on) {
            const int s = it / P, p = it - s * P;
            const T* qs = s_q + s * args.qstride;
            const int ip = qidx(0, p, rs);
            T* rec_out = s_beads + static_cast<int64_t>(it) * RL;
            T v[A2P];
            T qmax = T(0);
            if (on) {
                const int pn = (p + 1 == P) ? 0 : p + 1;
                const T* ql = kLo ? s_ql + s * args.qstride : nullptr;
                const int ipn = qidx(0, pn, rs);
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
                    if (QM != kQ32V)
#pragma unroll
                        for (int pr = 0; pr < A2; ++pr) v[pr] = fma(lr[pr], qa, v[pr]);
                }
                T lmax;
                {
#pragma unroll
                    for (int a = 0; a < A; ++a) {
#pragma unroll
                        for (int k = 0; k <= K; ++k) phv[k][a] -= dsum[k];
                        phr[a] -= rdsum;
                    }
                    lmax = phv[0][0];
#pragma unroll
                    for (int a = 1; a < A; ++a) lmax = max(lmax, phv[0][a]);
#pragma unroll
                    for (int a = 0; a < A; ++a)
                        if (a < nfill) lmax = max(lmax, phr[a]);
                    rec_out[OFF_L] = lmax;
#pragma unroll
                    for (int a = 0; a < A; ++a) rec_out[OFF_R + a] = (a < nfill) ? phr[a] - lmax : T(0);
                    T ob[OFF_L - OFF_O];                  // the O series block, row k = order k
#pragma unroll
                    for (int i = (K + 1) * A; i < OFF_L - OFF_O; ++i) ob[i] = T(0);
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
                        for (int k = 0; k <= K; ++k) ob[k * A + a] = e0 * ek[k];
                    }
                    // 128-bit stores where the block is float4-aligned (from 6 surfaces on)
                    stv(rec_out + OFF_O, ob);
                }
                if (QM == kQ32V) {
                    const float* vr = args.vq + ((base + s) * static_cast<int64_t>(P) + p) * args.vq_ld;
#pragma unroll
                    for (int pr = 0; pr < A2; pr += 4) {
                        const float4 w = *reinterpret_cast<const float4*>(vr + pr);
                        v[pr] = T(w.x);
                        if (pr + 1 < A2) v[pr + 1] = T(w.y);
                        if (pr + 2 < A2) v[pr + 2] = T(w.z);
                        if (pr + 3 < A2) v[pr + 3] = T(w.w);
                    }
                }
            }
            if constexpr (QM != kQ32V) {
                bool quad_done = false;
                if constexpr (kTcq) {
                    // tensor cores, unless a record of the warp has a coordinate beyond FP16's
                    // range for the products (then the FP32 loop over the global table)
                    if (!__any_sync(0xffffffffu, on && !(qmax <= T(kTcqMaxQ)))) {
                        int rec[4];
                        const int itw = it_base + (tid & ~31), nrec = nvalid * P;
#pragma unroll
                        for (int r = 0; r < 4; ++r) {
                            int ir = itw + 16 * (r >> 1) + 8 * (r & 1) + (lane >> 2);   // fragment rows: lane / 4 (+ 8)
                            ir = ir < nrec ? ir : 0;
                            const int sr = ir / P, pr_ = ir - sr * P;
                            rec[r] = plan.q + sr * args.qstride + qidx(0, pr_, rs);
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
            }
            if (on) {
                if constexpr (sizeof(T) == 4 && A >= kExpmMinA && A <= kTeamExpmMaxA) {
                    // M = exp(-tau V) by scaling and squaring in registers (see expm_neg_tau)
                    float vp[A2], X[A2], f;
#pragma unroll
                    for (int i = 0; i < A2; ++i) vp[i] = v[i];
                    rec_out[OFF_N] = T(expm_neg_tau_packed<A>(vp, static_cast<float>(m.tau), X, f));
                    T mo[OFF_O];
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c < A; ++c) mo[b * A + c] = f * X[sym_index(b, c)];
#pragma unroll
                    for (int i = A * A; i < OFF_O; ++i) mo[i] = T(0);
                    stv(rec_out, mo);
                } else {
                    T am[A][A], u[A][A];
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c <= b; ++c) { am[b][c] = v[pair_index(b, c)]; am[c][b] = am[b][c]; }
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c < A; ++c) u[b][c] = (b == c) ? T(1) : T(0);
                    jacobi_accumulate<T, A>(am, u, sizeof(T) == 4 ? 12 : 16);
                    T t[A];
                    T tmax = -tau_l2 * am[0][0];
#pragma unroll
                    for (int i = 0; i < A; ++i) { t[i] = -tau_l2 * am[i][i]; tmax = max(tmax, t[i]); }
                    const int n2 = static_cast<int>(floor(tmax));
                    rec_out[OFF_N] = T(n2);
                    T ev[A];
#pragma unroll
                    for (int i = 0; i < A; ++i) ev[i] = dev_exp2<T>(t[i] - T(n2));
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c <= b; ++c) {
                            T acc = T(0);
#pragma unroll
                            for (int i = 0; i < A; ++i) acc = fma(u[b][i] * ev[i], u[c][i], acc);
                            rec_out[b * A + c] = acc;
                            rec_out[c * A + b] = acc;
                        }
                }
            }
        };
        if constexpr (kTcq) {
            for (; it_base < nvalid * P; it_base += NT) {
                const int it = it_base + tid;
                record(it < nvalid * P ? it : 0, it < nvalid * P);
            }
        } else {
            for (int it = tid; it < nvalid * P; it += NT) record(it, true);
        }
        __syncthreads();

        // ================================ phase B2: row teams over bead chunks =================
        T nrow[K + 1][A];
        int nexp = 0;
        LogSum<T> lr, ls;
        const bool tact = team_ok && ts < nvalid;
        const int pb = tc * C, pe = min(P, pb + C);
        if (tact) {
#pragma unroll
            for (int k = 0; k <= K; ++k)
#pragma unroll
                for (int c = 0; c < A; ++c) nrow[k][c] = (k == 0 && c == r) ? T(1) : T(0);
            const T* recs = s_beads + static_cast<int64_t>(ts) * P * RL;
            for (int p = pb; p < pe; ++p) {
                const T* rc_ = recs + p * RL;
                nexp += static_cast<int>(rc_[OFF_N]);
                if (r == 0) ls.add(rc_[OFF_L]);
                if (r < A && r < nfill) lr.add(rc_[OFF_R + (r < A ? r : 0)]);
                if (r < A && kLeanB2) {
                    // column c of N M diag(O(c)): y = N(:, .) M(., c), then the series convolution
                    T nn[K + 1][A];
#pragma unroll
                    for (int c = 0; c < A; ++c) {
                        T mc[A], oc[K + 1];
#pragma unroll
                        for (int mm = 0; mm < A; ++mm) mc[mm] = rc_[mm * A + c];
#pragma unroll
                        for (int k = 0; k <= K; ++k) oc[k] = rc_[OFF_O + k * A + c];
                        if (p == pb) {
#pragma unroll
                            for (int k = 0; k <= K; ++k) {
                                T mrc = T(0);
#pragma unroll
                                for (int b = 0; b < A; ++b) mrc = (b == r) ? mc[b] : mrc;
                                nn[k][c] = mrc * oc[k];
                            }
                        } else {
                            T yc[K + 1];
#pragma unroll
                            for (int i = 0; i <= K; ++i) {
                                T acc = T(0);
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(nrow[i][mm], mc[mm], acc);
                                yc[i] = acc;
                            }
#pragma unroll
                            for (int k = 0; k <= K; ++k) {
                                T acc = T(0);
#pragma unroll
                                for (int i = 0; i <= k; ++i) acc = fma(yc[i], oc[k - i], acc);
                                nn[k][c] = acc;
                            }
                        }
                    }
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) nrow[k][c] = nn[k][c];
                } else if (r < A) {
                    T mf[OFF_O], of[OFF_L - OFF_O];         // from 6 surfaces whole 128-bit loads
                    ldv(rc_, mf);
                    ldv(rc_ + OFF_O, of);
                    T Mm[A][A], os[K + 1][A];
#pragma unroll
                    for (int b = 0; b < A; ++b)
#pragma unroll
                        for (int c = 0; c < A; ++c) Mm[b][c] = mf[b * A + c];
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) os[k][c] = of[k * A + c];
                    if (p == pb) {
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T mrc = T(0);
#pragma unroll
                                for (int b = 0; b < A; ++b) mrc = (b == r) ? Mm[b][c] : mrc;
                                nrow[k][c] = mrc * os[k][c];
                            }
                    } else {
                        T y[K + 1][A];
#pragma unroll
                        for (int i = 0; i <= K; ++i)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int mm = 0; mm < A; ++mm) acc = fma(nrow[i][mm], Mm[mm][c], acc);
                                y[i][c] = acc;
                            }
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int i = 0; i <= k; ++i) acc = fma(y[i][c], os[k - i][c], acc);
                                nrow[k][c] = acc;
                            }
                    }
                }
                if (((p - pb) & 1) == 1 || p + 1 == pe) {
                    // team-wide power-of-two renormalisation
                    T mx = T(0);
                    if (r < A) {
#pragma unroll
                        for (int c = 0; c < A; ++c) mx = max(mx, dev_fabs(nrow[0][c]));
                    }
#pragma unroll
                    for (int o = TA / 2; o >= 1; o >>= 1) mx = max(mx, __shfl_xor_sync(tmask, mx, o, TA));
                    if (mx > T(0) && isfinite(mx)) {
                        int e2;
                        frexp(mx, &e2);
                        const T sc = ldexp(T(1), -e2);
                        nexp += e2;
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) nrow[k][c] *= sc;
                    }
                }
            }
            if (pb >= pe) {
                // empty chunk: identity
#pragma unroll
                for (int k = 0; k <= K; ++k)
#pragma unroll
                    for (int c = 0; c < A; ++c) nrow[k][c] = (k == 0 && c == r) ? T(1) : T(0);
            }
        }
        __syncthreads();     // every thread is done reading bead records: the combine slots reuse them

        // ================================ phase C: combine chunks ==============================
        // Level st multiplies the chunk pairs (t0, t0 + st), t0 a multiple of 2 st, in bead order.
        // Split form (a second slot buffer fits and registers allow): all 2 st teams of the pair's
        // range work on its product, team u taking column group u of min(2 st, A) balanced groups,
        // thread r row r; products alternate between the two slot buffers (one barrier per level)
        // and the log sums and exponents merge in place (a pair's scalars are touched by one
        // thread).  The chunks enter normalised (max |N_0| in [1/2, 1)) and their products are not
        // renormalised: log2 G <= 5 levels move the entries by far less than the FP32 range, and
        // power-of-two scaling would not change a rounding.  Receiver form (the two-block build, or
        // no room): the team of chunk t0 multiplies its rows, held in registers, by its partner's
        // slot and renormalises.
        if (!kTwoBlock && plan.alt >= 0) {
            constexpr int CW = (A + 1) / 2;                        // most columns of one team
            T* comb = s_beads;
            T* comb_alt = sm + plan.alt;
            int* cexp = reinterpret_cast<int*>(s_lsum + S * G * (A + 1));
            const int slot = ts * G + tc;
            if (tact) {
                if (r < A)
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) comb[slot * CL + (k * A + r) * A + c] = nrow[k][c];
                if (r < A) s_lsum[slot * (A + 1) + r] = lr;
                if (r == 0) { s_lsum[slot * (A + 1) + A] = ls; cexp[slot] = nexp; }
            }
            __syncthreads();
            for (int st = 1; st < G; st <<= 1) {
                const int t0 = tc & ~(2 * st - 1), u = tc - t0;
                const int xs = ts * G + t0, ys = xs + st;
                const int ngrp = min(2 * st, A);
                if (tact && r < A && u < ngrp) {
                    const int c0 = (u * A) / ngrp, nc = ((u + 1) * A) / ngrp - c0;
                    const T* X = comb + xs * CL;
                    const T* Y = comb + ys * CL;
                    T* Z = comb_alt + xs * CL;
                    T xr[K + 1][A];
#pragma unroll
                    for (int i = 0; i <= K; ++i)
#pragma unroll
                        for (int mm = 0; mm < A; ++mm) xr[i][mm] = X[(i * A + r) * A + mm];
#pragma unroll
                    for (int cc = 0; cc < CW; ++cc) {
                        if (cc < nc) {
                            const int c = c0 + cc;
#pragma unroll
                            for (int k = 0; k <= K; ++k) {
                                T acc = T(0);
#pragma unroll
                                for (int i = 0; i <= k; ++i)
#pragma unroll
                                    for (int mm = 0; mm < A; ++mm) acc = fma(xr[i][mm], Y[((k - i) * A + mm) * A + c], acc);
                                Z[(k * A + r) * A + c] = acc;
                            }
                        }
                    }
                }
                if (tact && u == 0) {
                    if (r < A) {
                        LogSum<T> x = s_lsum[xs * (A + 1) + r];
                        x.merge(s_lsum[ys * (A + 1) + r]);
                        s_lsum[xs * (A + 1) + r] = x;
                    }
                    if (r == 0) {
                        LogSum<T> x = s_lsum[xs * (A + 1) + A];
                        x.merge(s_lsum[ys * (A + 1) + A]);
                        s_lsum[xs * (A + 1) + A] = x;
                        cexp[xs] += cexp[ys];
                    }
                }
                __syncthreads();
                T* sw = comb; comb = comb_alt; comb_alt = sw;
            }
            // the sample's product, log sums and exponent for phase D's team (tc == 0)
            if (tact && tc == 0 && G > 1) {
                const int s0 = ts * G;
                if (r < A) {
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) nrow[k][c] = comb[s0 * CL + (k * A + r) * A + c];
                    lr = s_lsum[s0 * (A + 1) + r];
                }
                if (r == 0) ls = s_lsum[s0 * (A + 1) + A];
                nexp = cexp[s0];
            }
        } else {
            T* comb = s_beads;
            int* cexp = reinterpret_cast<int*>(s_lsum + S * G * (A + 1));
            const int slot = ts * G + tc;
            if (tact) {
                if (r < A)
#pragma unroll
                    for (int k = 0; k <= K; ++k)
#pragma unroll
                        for (int c = 0; c < A; ++c) comb[slot * CL + (k * A + r) * A + c] = nrow[k][c];
                if (r < A) s_lsum[slot * (A + 1) + r] = lr;
                if (r == 0) { s_lsum[slot * (A + 1) + A] = ls; cexp[slot] = nexp; }
            }
            __syncthreads();
            for (int st = 1; st < G; st <<= 1) {
                const bool recv = tact && (tc % (2 * st)) == 0 && tc + st < G;
                if (recv) {
                    const int ps = slot + st;
                    const T* Y = comb + ps * CL;
                    if (r < A) {
                        T z[K + 1][A];
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) {
                                T acc = T(0);
#pragma unroll
                                for (int i = 0; i <= k; ++i)
#pragma unroll
                                    for (int mm = 0; mm < A; ++mm) acc = fma(nrow[i][mm], Y[((k - i) * A + mm) * A + c], acc);
                                z[k][c] = acc;
                            }
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) nrow[k][c] = z[k][c];
                        lr.merge(s_lsum[ps * (A + 1) + r]);
                    }
                    if (r == 0) ls.merge(s_lsum[ps * (A + 1) + A]);
                    nexp += cexp[ps];
                    T mx = T(0);
                    if (r < A) {
#pragma unroll
                        for (int c = 0; c < A; ++c) mx = max(mx, dev_fabs(nrow[0][c]));
                    }
#pragma unroll
                    for (int o = TA / 2; o >= 1; o >>= 1) mx = max(mx, __shfl_xor_sync(tmask, mx, o, TA));
                    if (mx > T(0) && isfinite(mx)) {
                        int e2;
                        frexp(mx, &e2);
                        const T sc = ldexp(T(1), -e2);
                        nexp += e2;
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) nrow[k][c] *= sc;
                    }
                    // own slot is no other receiver's partner at this level: write it back now
                    if (r < A)
#pragma unroll
                        for (int k = 0; k <= K; ++k)
#pragma unroll
                            for (int c = 0; c < A; ++c) comb[slot * CL + (k * A + r) * A + c] = nrow[k][c];
                    if (r < A) s_lsum[slot * (A + 1) + r] = lr;
                    if (r == 0) { s_lsum[slot * (A + 1) + A] = ls; cexp[slot] = nexp; }
                }
                __syncthreads();
            }
        }

        // ================================ phase D: outputs =====================================
        if (tact && tc == 0) {
            double coef[K + 1];
#pragma unroll
            for (int k = 0; k <= K; ++k) {
                // the trace summed in T across the team (the entries carry T's rounding already)
                T d = T(0);
#pragma unroll
                for (int c = 0; c < A; ++c) d = (c == r) ? nrow[k][c] : d;
                if (r >= A) d = T(0);
#pragma unroll
                for (int o = TA / 2; o >= 1; o >>= 1) d += __shfl_xor_sync(tmask, d, o, TA);
                coef[k] = scale_pow2(static_cast<double>(d), nexp);
            }
            const double lr_d = lr.value(), ls_d = ls.value();
            double rho = (r < A && r < nfill) ? exp_out<T>(lr_d) : 0.0;
#pragma unroll
            for (int o = TA / 2; o >= 1; o >>= 1) rho += __shfl_xor_sync(tmask, rho, o, TA);
            if (r == 0) {
                const int64_t sidx = base + ts;
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
        }
        __syncthreads();
    }
}

// MB: the blocks per SM the registers are sized for.  Two up to 4 surfaces; from 5 on one, plus a
// two-block build for 5 and 6 surfaces that the launcher picks when two tiles fit the shared memory
// of an SM (measured: +24-29 % at P = 32-64; at 7-8 surfaces the 128-register build spills and loses
// 10-13 %).
template <int A> constexpr int team_min_blocks() { return A <= 4 ? 2 : 1; }
constexpr int kTeamTwoBlockSmem = 113 * 1024;

// kTcq: the instantiation with B1's quadratic part of V on the tensor cores (launched when
// args.tcq is set; one block per SM only)
template <int A, int K, int QM, typename T, int MB = team_min_blocks<A>(), bool kTcq = false>
__global__ void __launch_bounds__(kTeamThreads, MB) pimc_team_kernel(const TeamArgs args) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sm = reinterpret_cast<T*>(smem_raw);
    const TeamPlan plan(A, K, QM, static_cast<int>(sizeof(T)), args.m.N, args.m.P, args.S, args.G,
                        args.qstride, args.rl, kTcq ? 1 : 0);
    team_load_tables<A, K, QM, T, kTcq>(args.m, args.rs, sm, plan);
    __syncthreads();
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * args.S; base < args.X;
         base += static_cast<int64_t>(gridDim.x) * args.S)
        team_tile<A, K, QM, T, MB, kTcq>(args, sm, plan, base);
}

// ---------------------------------------------------------------------------------------------
// Many independent models in one persistent launch (all with the same surface count A and series
// order K): the work is the concatenation of every model's tiles; CTAs take tiles round-robin,
// find the owning model by binary search over the tile prefix, and reload that model's tables
// into shared memory when it changes.  Each model keeps its own sizes (N, P), temperature, tile
// shape (S, G, C), seed, counter offset and outputs.
// ---------------------------------------------------------------------------------------------
struct TeamBatchItem {
    TeamArgs a;
    int64_t tile_begin;       // first tile of this model in the launch
};

template <int A, int K, int MB = team_min_blocks<A>(), bool kTcq = false>
__global__ void __launch_bounds__(kTeamThreads, MB)
pimc_team_batch_kernel(const TeamBatchItem* __restrict__ items, int n_items, int64_t total_tiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sm = reinterpret_cast<float*>(smem_raw);
    int cur = -1;
    TeamPlan plan;
    for (int64_t t = blockIdx.x; t < total_tiles; t += gridDim.x) {
        int lo = 0, hi = n_items - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
        }
        const TeamArgs& a = items[lo].a;
        if (lo != cur) {
            plan = TeamPlan(A, K, kSample, 4, a.m.N, a.m.P, a.S, a.G, a.qstride, a.rl, kTcq ? 1 : 0);
            team_load_tables<A, K, kSample, float, kTcq>(a.m, a.rs, sm, plan);
            __syncthreads();
            cur = lo;
        }
        team_tile<A, K, kSample, float, MB, kTcq>(a, sm, plan, (t - items[lo].tile_begin) * a.S);
    }
}

template <int A>
int launch_team(int K, int qmode, int precision, const TeamArgs& args, cudaStream_t stream);

template <int A>
int launch_team_batch(int K, const TeamBatchItem* items, int n_items, int64_t total_tiles, int smem_bytes,
                      int grid_cap, int tcq, cudaStream_t stream);

}  // namespace pbr
