/*
 * pibronic_gb300.h -- C ABI of the GB300 (sm_103a) PIMC block-evaluation library.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t (passed as void*),
 * is stream-ordered, allocates no device memory, and returns an int status (PBR_OK == 0).
 * The Python package pibronic_gb300 binds these with ctypes; any FFI can do the same.
 *
 * Reference path replaced: pibronic/pimc/pimc.py (the engine the reference README names
 * "pimc/minimal.py"), block loop pimc.py:1388-1462 and its stage functions pimc.py:1062-1213.
 */
#ifndef PIBRONIC_GB300_H
#define PIBRONIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ----------------------------------------------------------------------- */
#define PBR_OK              0
#define PBR_ERR_ARG         1   /* bad size / null pointer / unsupported shape              */
#define PBR_ERR_CUDA        2   /* a CUDA launch or runtime call failed                      */
#define PBR_ERR_UNSUPPORTED 3   /* no compiled variant for these sizes                       */
#define PBR_ERR_NONFINITE   4   /* a kernel produced a non-finite value (per-sample flag)   */
#define PBR_ERR_CAPACITY    5   /* request exceeds a fixed capacity of the library           */

/* ---- limits of the fused kernels ---------------------------------------------------------- */
#define PBR_MAX_A      8        /* surfaces of the coupled model                            */
#define PBR_MAX_A_RHO  16       /* surfaces of the sampling model                            */
#define PBR_MAX_N      64       /* modes                                                    */
#define PBR_MAX_P      1024     /* beads                                                    */
#define PBR_MAX_K      4        /* order of the beta series (0: g only; 4: g, g+ and g-)    */

/*
 * Device-resident model constants, built once per run on the host in FP64 by
 * pibronic_gb300.plan (the work BoxData.preprocess does, pimc.py:647-738) and uploaded.
 * All table pointers are device pointers to `precision`-bit floats (32: the production path;
 * 64: the FP64 validation path).  "pairs" are packed lower triangles (row >= col) in the order
 * (0,0),(1,0),(1,1),(2,0),... so pair(b,c) = b*(b+1)/2 + c for b >= c.  h is the step in beta.
 *
 *   vib_cs   [(K+1) * N]        1/2 x Taylor coefficients in h of csch(w_j (beta+h)/P)
 *   vib_th   [(K+1) * N]        1/2 x Taylor coefficients of tanh(w_j (beta+h)/(2P))
 *   vib_c    [(K+1) * A]        Taylor coefficients of ln prefactor_a(beta+h), minus log_c0 at k=0
 *                               (prefactor_a = exp(-tau Etilde_a) prod_j csch_j^(1/2), pimc.py:74-81)
 *   vib_d    [A * N]            state shift d_aj = -L_jaa / w_j  (pimc.py:212)
 *   vib_e    [A(A+1)/2]         off-diagonal energies (diagonal folded away, pimc.py:217)
 *   vib_l    [N * A(A+1)/2]     linear couplings, diagonal folded away (pimc.py:214)
 *   vib_qq   [N(N+1)/2 * A(A+1)/2]  for mode pair (d>=e): 1/2 (Q_de + Q_ed) if d>e, 1/2 Q_dd if d==e
 *   rho_cs, rho_th [N], rho_c [A_rho], rho_d [A_rho * N]   the sampling model at beta (order 0)
 *   mode_std [A_rho * N * P]    1/sqrt(2 coth_aj - csch_aj lambda_s) for ring normal mode s in
 *                               the real Fourier order: s=0 constant, s=2k-1 / 2k the cos / sin
 *                               pair of frequency k, s=P-1 the alternating mode when P is even
 *                               (pimc.py:402-404; any orthonormal eigenbasis of the ring gives
 *                               the same distribution of q)
 *   src_cdf  [A_rho]            cumulative normalised state weights       (pimc.py:343-350)
 *
 * The bead coordinates are x_pa = q_p - d_a and the O-matrix exponent is evaluated in the
 * cancellation-free form  coth (x_p^2 + x_p+1^2) - 2 csch x_p x_p+1
 *                       = csch (q_p - q_p+1)^2 + tanh(tau w / 2) (x_p^2 + x_p+1^2).
 */
typedef struct pbr_model {
    int32_t A, A_rho, n_fill_rho, N, P, K;
    int32_t precision;          /* 32 or 64: element type of every table below               */
    int32_t pad0;
    double  tau;                /* central beta / P; M = exp(-tau V) always uses it          */
    double  delta_beta;         /* beta step of the finite differences g(beta +- db)         */
    double  log_c0;             /* common offset removed from vib_c and rho_c at order 0     */
    const void* vib_cs;
    const void* vib_th;
    const void* vib_c;
    const void* vib_d;
    const void* vib_e;
    const void* vib_l;
    const void* vib_qq;
    const void* rho_cs;
    const void* rho_th;
    const void* rho_c;
    const void* rho_d;
    const void* mode_std;
    const void* src_cdf;
} pbr_model;

/*
 * Per-sample outputs of the fused path.  s_* are exactly the reference's result-file arrays
 * (BoxResultPM.scaled_rho / scaled_g / scaled_gofr_plus / scaled_gofr_minus, pimc.py:937-964):
 * products over beads divided by prod_p S12[p] (pimc.py:1076-1084).  g_coef[k] (optional) are the
 * Taylor coefficients of the scaled g(beta + h) in h, k = 0..K; log_scale (optional) is
 * ln prod_p S12[p] (add it back to recover the unscaled g and rho).  status (optional) gets
 * PBR_ERR_NONFINITE for a sample whose result is not finite.
 */
typedef struct pbr_outputs {
    double*  s_rho;             /* [X]                                                       */
    double*  s_g;               /* [X]                                                       */
    double*  s_gp;              /* [X]   nullable when K == 0                                */
    double*  s_gm;              /* [X]   nullable when K == 0                                */
    double*  g_coef;            /* [X * (K+1)]  nullable                                     */
    double*  log_scale;         /* [X]   nullable                                            */
    float*   q_out;             /* [X * N * P]  nullable: the sampled bead coordinates       */
    int32_t* src_out;           /* [X]   nullable: the sampled source surface                */
    int32_t* status;            /* [1]   nullable: max status over samples                   */
} pbr_outputs;

/*
 * Fused block evaluation with on-device sampling: draws X samples (Philox4x32-10 keyed by
 * seed, counter = offset + sample index), builds the O matrices of rho and of the coupled model
 * and its beta series, S12 scaling, V(q), Jacobi eigensolver, M = exp(-tau V), the ring product
 * with power-of-two log-scaling, and the traces.
 * Replaces one pass of the block loop of block_compute_pm / block_compute
 * (pimc.py:1413-1449 / 1358-1381), including draw_sample (pimc.py:326-334),
 * transform_sampled_coordinates (pimc.py:613-631), build_o_matrix (pimc.py:1087),
 * build_scaling_factors / scale_o_matrices (pimc.py:1062-1084), build_denominator
 * (pimc.py:1132), diagonalize_coupling_matrix (pimc.py:1139), build_numerator (pimc.py:1177).
 */
int pbr_sample_eval(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X,
                    const pbr_outputs* out, void* stream);

/*
 * Sampling only: the bead coordinates q [X * N * P] (FP32) and source surfaces src [X]
 * (nullable) that pbr_sample_eval draws for the same seed and offset.
 * Replaces draw_sample + transform_sampled_coordinates (pimc.py:326-334, 613-631).
 */
int pbr_sample_q(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X,
                 float* q_out, int32_t* src_out, void* stream);

/*
 * The same evaluation on caller-supplied bead coordinates q [X * N * P] (FP64, row-major
 * sample, mode, bead: the reference's qTensor[:, 0] layout, pimc.py:672).  Used for parity on
 * the reference's own samples and by the learned-proposal path.
 * Replaces pimc.py:1430-1449 for given data.qTensor (test_pimc_explicit_example.py:183-206).
 */
int pbr_eval_q(const pbr_model* model, const double* q, int64_t X, const pbr_outputs* out,
               void* stream);

/* As pbr_eval_q for FP32 bead coordinates (the learned proposal's samples). */
int pbr_eval_q_f32(const pbr_model* model, const float* q, int64_t X, const pbr_outputs* out,
                   void* stream);

/*
 * FP64 stage kernels: the reference's stage functions one by one, same layouts.
 *
 * pbr_o_matrix: O[B,P,Am,Am] dense, diagonal only, for q slots [B,Am,N,P];
 *   coth/csch [Am*N], shift [Am*N], prefactor [Am]; only the first n_fill diagonal entries set.
 *   Replaces build_o_matrix (pimc.py:1087-1129).
 */
int pbr_o_matrix(const double* q_slots, int64_t B, int32_t Am, int32_t N, int32_t P,
                 const double* coth, const double* csch, const double* shift,
                 const double* prefactor, int32_t n_fill, double* O, void* stream);

/* S12[B,P] = max over both O's, then O1, O2 (and O3..: extra, nullable) divided by it.
 * Replaces build_scaling_factors + scale_o_matrices (pimc.py:1062-1084, 1443, 1448). */
int pbr_scale_o_matrices(double* O1, int32_t A1, double* O2, int32_t A2, int64_t B, int32_t P,
                         double* S12, void* stream);

/* O[B,P,A,A] /= S12[B,P] (pimc.py:1443). */
int pbr_divide_o_matrix(double* O, int32_t A, int64_t B, int32_t P, const double* S12,
                        void* stream);

/* rho[idx] = Tr prod_p O[b,p]  (diagonal O).  Replaces build_denominator (pimc.py:1132-1136). */
int pbr_denominator(const double* O, int64_t B, int32_t A, int32_t P, double* out, void* stream);

/* V[B,P,A,A] from q slots, E[A*A], L[N*A*A], Q[N*N*A*A]; eigenvalues ascending [B,P,A] and
 * eigenvectors (columns) [B,P,A,A] by cyclic Jacobi in FP64 on the lower triangle; symmetric
 * flag (1 if V is symmetric to the reference's np.allclose) in *sym_ok.
 * Replaces diagonalize_coupling_matrix (pimc.py:1139-1174). */
int pbr_coupling_eigh(const double* q_slots, int64_t B, int32_t A, int32_t N, int32_t P,
                      const double* E, const double* L, const double* Q, double* V,
                      double* eigvals, double* eigvecs, int32_t* sym_ok, void* stream);

/* M = U diag(exp(-tau lambda)) U^T, then out[idx] = Tr prod_p (M_p O_p) for dense O.
 * Replaces build_numerator (pimc.py:1177-1213). */
int pbr_numerator(const double* eigvals, const double* eigvecs, const double* O, int64_t B,
                  int32_t A, int32_t P, double tau, double* M, double* out, void* stream);

/*
 * Device reduction of the per-sample outputs into the estimator moments (FP64; per-thread
 * Welford updates merged pairwise with Chan's formula, in a fixed order, so the result does not
 * depend on scheduling):
 *   moments[0..6] = n, mean r, M2 r, mean s1, M2 s1, mean s2, M2 s2   (M2 = sum of squared
 *   deviations from the mean), with r = g/rho, s1 = (g+ - g-)/(2 db rho),
 *   s2 = (g+ - 2g + g-)/(db^2 rho) (stats.py:38-55).  Z = mean r and its error
 *   sqrt(M2 r / n) / sqrt(n - 1) (stats.py:84-90), E = -mean s1 / Z, Cv = (mean s2 / Z - E^2)/(kB T^2).
 * scratch must hold 9 * pbr_reduce_blocks(X) doubles.
 * Replaces the numpy reductions of stats.estimate_basic_properties (stats.py:84-123).
 */
int pbr_reduce_terms(const double* s_rho, const double* s_g, const double* s_gp,
                     const double* s_gm, int64_t X, double delta_beta, double* scratch,
                     double* moments, void* stream);

/*
 * Jackknife second pass (jackknife.py:60-105).  With the totals S_r, S_1, S_2 of r, s1, s2 and
 * E0 = -S_1/S_r, the leave-one-out estimators are
 *   f_E,i = -(S_1 - s1_i)/(S_r - r_i),  f_C,i = ((S_2 - s2_i)/(S_r - r_i) - f_E,i^2)/(kB T^2).
 * The kernel reduces their deviations from the full-sample values, written without the
 * cancellation of the direct difference:
 *   dE_i = f_E,i - E0 = (S_r s1_i - S_1 r_i) / (S_r (S_r - r_i))
 *   dC_i = f_C,i - C0 = (-(S_r s2_i - S_2 r_i) / (S_r (S_r - r_i)) - dE_i (2 E0 + dE_i)) / (kB T^2)
 * into out[0..4] = n, mean dE, M2 dE, mean dC, M2 dC (same merge as pbr_reduce_terms).
 * totals = {S_r, S_1, S_2}.  scratch must hold 6 * pbr_reduce_blocks(X) doubles.
 */
int pbr_reduce_jackknife(const double* s_rho, const double* s_g, const double* s_gp,
                         const double* s_gm, int64_t X, double delta_beta, double kB_T2,
                         const double* totals, double* scratch, double* out, void* stream);

/* Number of partial blocks the reductions use for X samples. */
int64_t pbr_reduce_blocks(int64_t X);

/*
 * pbr_reduce_terms without a scratch argument: allocates nothing and takes no scratch buffer.
 * No counterpart in the reference.  It is for callers that cannot allocate device memory -- a
 * plain FFI caller with no GPU array library to allocate through, or one whose device memory is
 * held by its own pool and that must not call cudaMalloc/cudaFree (they can synchronize the
 * device).  The partial sums live in a fixed file-scope device array of 9 * 1024 doubles
 * (72 KiB) that every device loading the library keeps until the process exits, so
 * X <= pbr_reduce_terms_static_max_samples() = 4,194,304; larger X returns PBR_ERR_CAPACITY and
 * launches nothing.  Results equal pbr_reduce_terms's for the same inputs.  The first call on a
 * device looks the array's device address up (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  All calls share the one array: calls that
 * overlap on the GPU (other streams, other host threads) race and must be serialised by the
 * caller.
 */
int pbr_reduce_terms_static(const double* s_rho, const double* s_g, const double* s_gp,
                            const double* s_gm, int64_t X, double delta_beta, double* moments,
                            void* stream);
int64_t pbr_reduce_terms_static_max_samples(void);

/*
 * FP32 FMA throughput probe: blocks x 256 threads, each running 8 independent FMA chains for
 * 16 * iters steps; *flops gets the flop count of the launch.  Time it with events to get the
 * CUDA-core FP32 peak the fused kernel is compared against.  No counterpart in the reference
 * (a measurement utility).
 */
int pbr_fma_probe(float* out, int32_t blocks, int32_t iters, double* flops, void* stream);

/* Library version string and the SM architecture it was built for. */
const char* pbr_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PIBRONIC_GB300_H */
