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
#define PBR_MAX_A      8        /* surfaces of the coupled model (fused kernels)            */
#define PBR_MAX_A_WIDE 16       /* surfaces of the coupled model (pbr_sample_eval_tc)        */
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
 *   ring_chol [3 * P * N]       per mode j, the bead precision of rho, 2 coth_j I - csch_j C
 *                               (C the ring adjacency; pimc.py:402-404), factored L L^T: a_p =
 *                               1/L_pp, b_p = L_{p+1,p} (L_{P-1,P-2} at p = P-2), c_p = L_{P-1,p}
 *                               (p <= P-3), as bead-major arrays a[p][j], b[p][j], c[p][j].  The matrix is
 *                               cyclic tridiagonal, so L is bidiagonal plus a dense last row and
 *                               q - d = L^-T z (z standard normal) costs O(P) per mode.
 *   src_cdf  [A_rho]            cumulative normalised state weights       (pimc.py:343-350)
 *
 * The bead coordinates are x_pa = q_p - d_a and the O-matrix exponent is evaluated in the
 * cancellation-free form  coth (x_p^2 + x_p+1^2) - 2 csch x_p x_p+1
 *                       = csch (q_p - q_p+1)^2 + tanh(tau w / 2) (x_p^2 + x_p+1^2).
 */
typedef struct pbr_model {
    int32_t A, A_rho, n_fill_rho, N, P, K;
    int32_t precision;          /* 32 or 64: element type of every table below               */
    int32_t variant;            /* fused-kernel form: 0 auto, 1 register chunks (A <= 4),
                                   2 bead-parallel + row teams (A <= 8)                       */
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
    const void* ring_chol;
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
 * seed, counter = offset + sample index; the source surface from the state weights, then for each
 * mode q - d_src = L^-T z by back substitution), builds the O matrices of rho and of the coupled model
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
 * The same block evaluation with the potential V(q) built on the tensor cores, for large N
 * (precision 32 only): per chunk of samples the sampler writes q (into out->q_out when given,
 * else into scratch), the tcgen05 GEMM (FP16, hi/lo split, three MMAs per K step) writes V for
 * every (sample, bead) row, and the row-team kernel evaluates the chunk from q and that V.  Draws the same samples as pbr_sample_eval for the same seed and
 * offset.  scratch (256-byte aligned, scratch_bytes long) bounds the chunk:
 * pbr_sample_eval_tc_scratch(model, chunk) is the size for a chunk of that many samples; a
 * scratch too small for one sample gives PBR_ERR_CAPACITY.  Replaces the same reference stages
 * as pbr_sample_eval (V is pimc.py:1145-1150).
 */
int64_t pbr_sample_eval_tc_scratch(const pbr_model* model, int64_t chunk);
int pbr_sample_eval_tc(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X,
                       const pbr_outputs* out, void* scratch, int64_t scratch_bytes, void* stream);

/* As pbr_sample_eval_tc on caller-supplied FP32 bead coordinates q [X * N * P] (the learned
 * proposal's samples at large N or more than 8 surfaces); the sampler stage is skipped.
 * Replaces pimc.py:1430-1449 for given data.qTensor, as pbr_eval_q_f32. */
int pbr_eval_q_tc(const pbr_model* model, const float* q, int64_t X, const pbr_outputs* out,
                  void* scratch, int64_t scratch_bytes, void* stream);

/*
 * Many independent models in one launch per surface count (the batched configuration): every
 * model keeps its own sizes, temperature, seed, counter offset and outputs.  pbr_batch_pack fills
 * a host blob of pbr_batch_blob_bytes(n) bytes; smem_budgets (nullable; entries 0..8, indexed by
 * the surface count) chooses each group's kernel form and tile shape: < 0 one register-chunk
 * launch per model (up to 4 surfaces, the faster form there as a rule), 0 the row-team form with
 * tiles sized for the whole shared memory, > 0 the row-team form with tiles within that many
 * bytes (a model whose one-sample tile exceeds the budget takes the whole shared memory instead);
 * a null table means register chunks up to 4 surfaces and whole-memory row-team tiles beyond.
 * Models group by surface count and series order (and at 5-6 surfaces by whether two tiles fit an
 * SM); grid_cap limits the persistent grid, 0 = occupancy x SMs.  The caller copies the blob to a
 * device buffer of the same size; pbr_sample_eval_batch launches one persistent row-team kernel
 * per row-team group, CTAs taking the concatenated tiles round-robin, and the register-chunk
 * launches of the other groups.  All models need precision 32.  The launches can be captured in a
 * CUDA graph (the blob holds everything they read).
 */
int64_t pbr_batch_blob_bytes(int32_t n_models);
int pbr_batch_pack(const pbr_model* models, const uint64_t* seeds, const uint64_t* offsets, const int64_t* X,
                   const pbr_outputs* outs, int32_t n_models, const int32_t* smem_budgets, int32_t grid_cap,
                   void* host_blob);
int pbr_sample_eval_batch(const void* host_blob, const void* device_blob, void* stream);
int32_t pbr_batch_groups(const void* host_blob);

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

/* S1[B,P] = max over O1[b,p], S2[B,P] = max over O2[b,p] (S1, S2 nullable), S12 = max(S1, S2).
 * Replaces build_scaling_factors (pimc.py:1076-1084). */
int pbr_scaling_factors(const double* O1, int32_t A1, const double* O2, int32_t A2, int64_t B, int32_t P,
                        double* S1, double* S2, double* S12, void* stream);

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

/*
 * Segmented forms for batched launches: M independent reductions over s_*[seg[m] .. seg[m+1])
 * (seg: M+1 int64, device), each with its own delta_beta[m] (and kB T^2 [m]); moments [M][7] and
 * out [M][5] in the layouts above; the jackknife pass takes the moments of the first.  scratch
 * holds pbr_reduce_segments_scratch(M) doubles.  M <= 65535.
 */
int pbr_reduce_terms_segments(const double* s_rho, const double* s_g, const double* s_gp, const double* s_gm,
                              const int64_t* seg, int32_t M, const double* delta_beta, double* scratch,
                              double* moments, void* stream);
int pbr_reduce_jackknife_segments(const double* s_rho, const double* s_g, const double* s_gp, const double* s_gm,
                                  const int64_t* seg, int32_t M, const double* delta_beta, const double* kB_T2,
                                  const double* moments, double* scratch, double* out, void* stream);
int64_t pbr_reduce_segments_scratch(int32_t M);

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
 * make that first call before any stream capture.  The address is kept for the life of the
 * process: a cudaDeviceReset (or any release and re-creation of the device's primary context)
 * can move the array, so after one this entry point must not be called again on that device in
 * the same process.  All calls share the one array: calls that
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

/* ============================================================================================
 * Learned importance proposal (affine-coupling flow over whitened ring normal modes).
 * No counterpart in the reference: Pibronic's learned-proposal seam only produces training data
 * (block_compute_gR*, pimc.py:1216-1338); these kernels train and apply the proposal on the GPU.
 * All arrays are FP32 unless stated, row-major, device pointers.
 * ============================================================================================ */

/* One coupling layer: D coordinates split into I conditioning (idx_a) and J transformed (idx_b)
 * positions; conditioner tanh(tanh(y_A W1 + b1) W2 + b2) W3 + b3 with W1 [I][H], W2 [H][H],
 * W3 [H][2J] (the first J outputs give s = 2 tanh(raw/2), the last J give t). */
typedef struct pbr_flow_layer {
    int32_t D, I, J, H;
    const int32_t* idx_a;
    const int32_t* idx_b;
    const float* W1; const float* b1;
    const float* W2; const float* b2;
    const float* W3; const float* b3;
} pbr_flow_layer;

/* Activations a training pass keeps per layer: ya [X][I], h1 / h2 [X][H], s / yb [X][J]. */
typedef struct pbr_flow_save {
    float* ya; float* h1; float* h2; float* s; float* yb;
} pbr_flow_save;

/* y [X][N*nsel] = whitened ring normal-mode slots s < nsel of q - center (center [N] FP64,
 * inv_sigma [N*nsel] FP64 = sqrt(2 coth - csch lambda_s)); U [X] (FP64) = the rest of rho's
 * bead quadratic form sum_j (q_j - c_j)^T Lambda_j (q_j - c_j) - |y|^2 (rho_csch [N],
 * rho_tanh2 [N] = tanh(tau w / 2), FP64).  nsel <= 8. */
int pbr_flow_prepare(const float* q, int64_t X, int32_t N, int32_t P, int32_t nsel, const double* center,
                     const double* inv_sigma, const double* rho_csch, const double* rho_tanh2, float* y,
                     double* U, void* stream);

/* x = q + sum_{s<nsel} B_ps sigma_js (y_new - y)_js  (sigma [N*nsel] FP64). */
int pbr_flow_apply(const float* q, const float* y, const float* y_new, int64_t X, int32_t N, int32_t P,
                   int32_t nsel, const double* sigma, float* x, void* stream);

/* One coupling layer in place on y [X][D]; direction +1 (sampling: y_B e^s + t, logdet += sum s)
 * or -1 (density: (y_B - t) e^-s, logdet -= sum s); logdet [X] FP64; save nullable. */
int pbr_flow_layer_forward(const pbr_flow_layer* layer, int32_t direction, int64_t X, float* y,
                           double* logdet, const pbr_flow_save* save, void* stream);

/* The same layer in the sampling direction (+1) on the tensor cores: per tile of 128 samples the
 * three products as tcgen05.mma kind::f16 GEMMs with BF16 weights and activations and FP32
 * accumulation in TMEM; the coupling update y_B e^s + t and logdet += sum s in FP32 (logdet FP64).
 * The log-determinant is exactly that of the map applied (y_A passes unchanged), so the proposal
 * density stays exact for the BF16 network.  pbr_flow_tc_pack converts the layer's FP32 weights
 * into `packed` (pbr_flow_tc_packed_bytes(D, I, J, H) bytes, 16-byte aligned; -1 when the shape
 * is unsupported: H a multiple of 32 up to 128, I <= 128, 2J <= 256, and the packed weights with
 * one 128-sample tile of y within 227 KB of shared memory); repack after the weights
 * change.  status (nullable) gets PBR_ERR_CUDA if a bounded wait gave up.  No counterpart in the
 * reference. */
int64_t pbr_flow_tc_packed_bytes(int32_t D, int32_t I, int32_t J, int32_t H);
int pbr_flow_tc_pack(const pbr_flow_layer* layer, void* packed, void* stream);
int pbr_flow_tc_forward(const pbr_flow_layer* layer, const void* packed, int64_t X, float* y, double* logdet,
                        int32_t* status, void* stream);

/* Back-propagation through one layer of the -1 direction using its saved activations:
 * gy [X][D] holds dL/d(output) on entry, dL/d(input) on exit; rt [X] the per-sample weights of
 * the log-det term; writes g_o [X][2J], g_z2 [X][H], g_z1 [X][H] for the weight gradients. */
int pbr_flow_layer_backward(const pbr_flow_layer* layer, int64_t X, float* gy, const float* rt,
                            const pbr_flow_save* save, float* g_o, float* g_z2, float* g_z1, void* stream);

/* C [M][N] = beta C + sum_x A[x][M] B[x][N] (C is not read when beta == 0) and, when colsum is
 * not NULL, colsum [N] = sum_x B[x][N] (the bias gradient that shares the B operand), split over
 * the batch and reduced in a fixed order; scratch holds pbr_gemm_tn_scratch(X, M, N) floats. */
int pbr_gemm_tn_acc(const float* A, const float* B, int64_t X, int32_t M, int32_t N, float beta, float* C,
                    float* colsum, float* scratch, void* stream);
int64_t pbr_gemm_tn_scratch(int64_t X, int32_t M, int32_t N);

/* out [N] = column sums of B [X][N]. */
int pbr_colsum(const float* B, int64_t X, int32_t N, float* out, void* stream);

/* Base mixture on y0 [X][D]: lse [X] (FP64, nullable) = log sum_a exp(log_pi_a - |y0 - mu_a|^2/2);
 * with rt: gy [X][D] = rt sum_a gamma_a (y0 - mu_a), rgam [X][A] = rt gamma, lossterm [X] (FP64)
 * = -rt (lse + ld) (ld [X] FP64).  Outputs nullable.  A <= 16. */
int pbr_flow_base(const float* y0, const double* ld, int64_t X, int32_t D, int32_t A, const float* mu,
                  const float* log_pi, const float* rt, float* gy, float* rgam, double* lossterm,
                  double* lse, void* stream);

/* s_q [X] = exp(lse_y - U/2 - logdet - log_scale_x) (all FP64): the proposal density of the
 * flowed sample in the scale of its PIMC outputs (pbr_outputs.log_scale). */
int pbr_flow_weights(const double* lse_y, const double* U, const double* logdet, const double* log_scale_x,
                     int64_t X, double* s_q, void* stream);

/* Adam step: *step (device int32) is incremented first and the update is bias-corrected with the
 * new value, so the call can be replayed from a captured CUDA graph. */
int pbr_adam(float* param, const float* grad, float* m, float* v, int64_t n, float lr, float beta1,
             float beta2, float eps, int32_t* step, void* stream);

/*
 * 5th-generation tensor-core GEMM (tcgen05.mma into TMEM, operands staged in shared memory in the
 * no-swizzle K-major core-matrix layout, completion through an mbarrier, tcgen05.ld epilogue):
 * C [M][N] FP32 = A [M][K] B [N][K]^T with fmt 1 = BF16 or 2 = TF32 (FP32 storage) operands,
 * M % 128 == 0, N % 16 == 0 and 16 <= N <= 256, K a multiple of 64 (BF16) or 32 (TF32), A and B
 * 16-byte aligned.  Waits are bounded: a CTA that times out writes PBR_ERR_CUDA to *status
 * (nullable) and frees its tensor memory.  No counterpart in the reference (the contraction the
 * reference does with numpy einsum, pimc.py:1147, at large N).
 */
int pbr_tc_gemm(int32_t fmt, const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K,
                int32_t* status, void* stream);

/*
 * The diabatic potential alone (the middle stage of pbr_sample_eval_tc), for tests and custom
 * pipelines: V(q) = E + sum_j L_j q_j + sum_{d >= e} Qp_de q_d q_e as one tcgen05 GEMM
 * (kind::f16: FP16 hi/lo split of both operands after exact power-of-two scaling of each bead row
 * and of the couplings, three MMAs per K step of 16, FP32 accumulation in TMEM, about 22 bits
 * per product).  K is laid out in quads of four columns (d, e0..e0+3) over the bead row's slots
 * s = [q_0..q_{N-1}, 0 up to NA = N rounded up to 4, 1, 0, 0, 0]: quads (d < N, e0 = 0, 4, .. <= d)
 * hold the pairs e <= d, quads (NA, j0) the linear terms, quad (NA, NA) the energies, quads
 * (NA + 1, NA) pad to a multiple of 64.
 * pbr_tc_potential_dims gives the padded K extent n2p and the column count a2p (A(A+1)/2 rounded up
 * to 16).  pbr_tc_pack_potential turns vib_qq [N(N+1)/2][A(A+1)/2], vib_l [N][A(A+1)/2] and vib_e
 * [A(A+1)/2] (FP32 or FP64 as precision says; vib_l and vib_e nullable = zero) into b_packed
 * (pbr_tc_potential_packed_floats(N, A) = a2p * n2p + 4 32-bit words, 16-byte aligned): per stage
 * of 64 K columns, the FP16 hi part then the lo part of the couplings times 2^s_B, each a2p rows x
 * 8 cores of 8 columns, core (row r, core c) at ((r/8)*8 + c)*8 + r%8 in 16-byte units; row
 * A(A+1)/2 (the first padding row) holds 1 at the energies' column; then the largest |coupling|
 * and the FP32 scale 2^s_B (the largest scaled coupling is below 2^14).
 * pbr_tc_potential writes vq [X * P][a2p] (FP32; row sample * P + bead, column pair_index(b, c))
 * from q [X][N][P] (FP32).  A <= 16, N <= 64.  Waits are bounded as in pbr_tc_gemm.  Replaces
 * pimc.py:1145-1150 (V of diagonalize_coupling_matrix).
 */
/* Tensor-pipe rate: one CTA per SM issues reps back-to-back tcgen05.mma from one thread --
 * fmt 2: kind::tf32, M x N x 8; fmt 1: kind::f16 with BF16 operands, M x N x 16 (M 64 or 128,
 * 16 <= N <= 256) -- round-robin over nacc (1..4) independent TMEM accumulators, A from shared
 * memory or (a_tmem = 1, M = 128) from TMEM; *tflops is the whole-GPU rate,
 * *cycles_per_mma the issuing thread's cycles per instruction.  scratch: 16 bytes of the caller's
 * device memory, 8-byte aligned (the cycle count and the kernel's wait flag).  Synchronizes the
 * stream to read the result (a measurement, not a path entry point).  No counterpart in the
 * reference. */
int pbr_tc_mma_rate(int32_t fmt, int32_t M, int32_t N, int32_t nacc, int32_t a_tmem, int32_t reps, void* scratch,
                    double* tflops, double* cycles_per_mma, void* stream);

int pbr_tc_potential_dims(int32_t N, int32_t A, int32_t* n2p, int32_t* a2p);
int64_t pbr_tc_potential_packed_floats(int32_t N, int32_t A);
int pbr_tc_pack_potential(const void* vib_qq, const void* vib_l, const void* vib_e, int32_t precision,
                          int32_t N, int32_t A, void* b_packed, void* stream);
int pbr_tc_potential(const float* q, int64_t X, int32_t N, int32_t P, int32_t A, const void* b_packed,
                     float* vq, int32_t* status, void* stream);

/* Library version string and the SM architecture it was built for. */
const char* pbr_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PIBRONIC_GB300_H */
