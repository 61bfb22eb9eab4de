// pbr_api.cu -- extern "C" entry points of the fused path (declared in include/pibronic_gb300.h).
#include <algorithm>
#include <cstring>

#include "pbr_team.cuh"
#include "pbr_wide.cuh"

namespace pbr {
template <int A> int launch_fused(int, int, int, const FusedArgs&, cudaStream_t);
template <int A> int launch_team(int, int, int, const TeamArgs&, cudaStream_t);
template <int A> int launch_team_batch(int, const TeamBatchItem*, int, int64_t, int, int, int, cudaStream_t);
int tc_quadratic_cols(int A);
int tc_quadratic_kdim(int N);
int64_t tc_packed_floats(int N, int A);
int tc_quadratic_launch(const float*, int64_t, int, int, int, const void*, float*, int32_t*, cudaStream_t);
int tc_pack_launch(const void*, const void*, const void*, int, int, int, void*, cudaStream_t);
extern template int launch_wide<12>(int, const WideArgs&, cudaStream_t);   // pbr_wide_a12.cu
extern template int launch_wide<16>(int, const WideArgs&, cudaStream_t);   // pbr_wide_a16.cu
extern template int wide_resident<12>(int, const WideArgs&);
extern template int wide_resident<16>(int, const WideArgs&);
}

namespace {

constexpr int kMaxSmem = 227 * 1024;   // opt-in shared memory per CTA on sm_103a

int pow2ceil(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

int ilog2(int x) {
    int l = 0;
    while ((1 << l) < x) ++l;
    return l;
}

// Row stride of the row-team kernel's q block.  For a model that can take the tensor-core
// quadratic (FP32, 5-8 surfaces, from kTcqMinN modes) the stride is raised to the nearest residue
// 10, 14, 18 or 22 mod 32: each MMA fragment load reads 8 consecutive beads at the mode offsets of
// 4 mode quadruples, and those residues spread the 32 reads over the fewest banks for every mode
// count from 16 to 64 (1.3-1.4 wavefronts per read, against 1.6-2.6 at the residues 2, 4 and 8
// that row_stride gives at P = 64, 128 and 256).  Residues 2 mod 4 also keep the sampler's
// per-(sample, mode) chains, which run side by side over consecutive modes, at 2-way conflicts.
int team_row_stride(const pbr_model& m) {
    int rs = pbr::row_stride(m.P);
    if (m.precision != 32 || m.A < 5 || m.A > 8 || m.N < pbr::kTcqMinN) return rs;
    while (!((rs & 31) == 10 || (rs & 31) == 14 || (rs & 31) == 18 || (rs & 31) == 22)) ++rs;
    return rs;
}

// Tile shape of the row-team form for one model: S samples per tile (as many as 256 threads
// hold, halved until the shared memory fits the budget), G teams per sample, C beads per team.
int make_team_args(const pbr_model& m, int qmode, const void* q_in, int64_t X, uint64_t seed,
                   uint64_t offset, const pbr_outputs* out, int smem_budget, pbr::TeamArgs* pa) {
    using namespace pbr;
    TeamArgs& a = *pa;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    a.q_in = q_in;
    a.X = X;
    a.out = *out;
    a.key0 = static_cast<uint32_t>(seed);
    a.key1 = static_cast<uint32_t>(seed >> 32);
    a.offset = offset;
    a.rs = team_row_stride(m);
    a.qstride = m.N * a.rs + 1;
    a.rl = record_len(m.A, m.K);
    const int esz = m.precision == 32 ? 4 : 8;
    const int TA = pow2_ceil(m.A);
    const int max_teams = kTeamThreads / TA;
    a.S = std::max(1, kTeamThreads / m.P);
    while (true) {
        // teams per sample: the largest power of two that the threads hold and the ring can use
        a.G = 1;
        while (a.G * 2 <= max_teams / a.S && a.G * 2 <= m.P) a.G *= 2;
        const TeamPlan plan(m.A, m.K, qmode, esz, m.N, m.P, a.S, a.G, a.qstride, a.rl);
        if (plan.total_bytes <= smem_budget) break;
        if (a.S == 1) return PBR_ERR_UNSUPPORTED;
        a.S = std::max(1, a.S / 2);
    }
    a.C = (m.P + a.G - 1) / a.G;
    return PBR_OK;
}

int team_smem(const pbr::TeamArgs& a, int qmode) {
    const pbr::TeamPlan plan(a.m.A, a.m.K, qmode, a.m.precision == 32 ? 4 : 8, a.m.N, a.m.P, a.S, a.G,
                             a.qstride, a.rl, a.tcq);
    return plan.total_bytes;
}

// B1's tensor-core quadratic for a single-model row-team launch: FP32, q drawn or given (not V),
// 5-8 surfaces (one block per SM; the two-block build at 5-6 surfaces is kept when its tile
// fits), from kTcqMinN modes, and only when its tables still fit the budget
void choose_team_tcq(pbr::TeamArgs& a, int qmode, int smem_budget) {
    using namespace pbr;
    a.tcq = 0;
    const pbr_model& m = a.m;
    if (m.precision != 32 || qmode == kQ32V || m.A < 5 || m.A > 8 || m.N < kTcqMinN) return;
    if ((m.A == 5 || m.A == 6) && team_smem(a, qmode) <= kTeamTwoBlockSmem) return;
    a.tcq = 1;
    const TeamPlan pt(m.A, m.K, qmode, 4, m.N, m.P, a.S, a.G, a.qstride, a.rl, 1);
    if (pt.tcq_k == 0 || pt.total_bytes > smem_budget) a.tcq = 0;
}

int run_team(const pbr_model& m, int qmode, const void* q_in, int64_t X, uint64_t seed,
             uint64_t offset, const pbr_outputs* out, cudaStream_t st, const float* vq = nullptr,
             int vq_ld = 0) {
    using namespace pbr;
    TeamArgs a;
    const int rc = make_team_args(m, qmode, q_in, X, seed, offset, out, kMaxSmem, &a);
    if (rc != PBR_OK) return rc;
    choose_team_tcq(a, qmode, kMaxSmem);
    a.vq = vq;
    a.vq_ld = vq_ld;
    switch (m.A) {
        case 1: return launch_team<1>(m.K, qmode, m.precision, a, st);
        case 2: return launch_team<2>(m.K, qmode, m.precision, a, st);
        case 3: return launch_team<3>(m.K, qmode, m.precision, a, st);
        case 4: return launch_team<4>(m.K, qmode, m.precision, a, st);
        case 5: return launch_team<5>(m.K, qmode, m.precision, a, st);
        case 6: return launch_team<6>(m.K, qmode, m.precision, a, st);
        case 7: return launch_team<7>(m.K, qmode, m.precision, a, st);
        case 8: return launch_team<8>(m.K, qmode, m.precision, a, st);
        default: return PBR_ERR_UNSUPPORTED;
    }
}

int check_model(const pbr_model& m, int qmode, const void* q_in, const pbr_outputs* out, int max_a = PBR_MAX_A) {
    using namespace pbr;
    if (m.A < 1 || m.A > max_a) return PBR_ERR_UNSUPPORTED;
    if (m.variant < 0 || m.variant > 3) return PBR_ERR_ARG;
    if (m.A_rho < m.A || m.A_rho > PBR_MAX_A_RHO) return PBR_ERR_ARG;
    if (m.n_fill_rho != m.A) return PBR_ERR_ARG;
    if (m.N < 1 || m.N > PBR_MAX_N || m.P < 3 || m.P > PBR_MAX_P) return PBR_ERR_ARG;
    if (m.K != 0 && m.K != 4) return PBR_ERR_UNSUPPORTED;
    if (m.precision != 32 && m.precision != 64) return PBR_ERR_ARG;
    if (!out->s_rho || !out->s_g) return PBR_ERR_ARG;
    if (m.K > 0 && (!out->s_gp || !out->s_gm)) return PBR_ERR_ARG;
    if (!m.vib_cs || !m.vib_th || !m.vib_c || !m.vib_d || !m.vib_e || !m.vib_l || !m.vib_qq ||
        !m.rho_cs || !m.rho_th || !m.rho_c || !m.rho_d)
        return PBR_ERR_ARG;
    if (qmode == kSample && (!m.ring_chol || !m.src_cdf)) return PBR_ERR_ARG;
    if (qmode != kSample && !q_in) return PBR_ERR_ARG;
    return PBR_OK;
}

// Per-sample stride of the register-chunk kernel's q block: N rows of rs floats plus a pad in
// [1, 32].  A warp holds 32 / G samples x G bead chunks of C beads, and each bead step reads the
// same mode of all of them (the O series, the linear and the quadratic part of V); the pad is the
// smallest that spreads those 32 reads over the fewest wavefronts, summed over the chunk's steps
// (at A = 4, N = 12, P = 64 a pad of 1 put two pairs of lanes in one bank on every read, 2
// wavefronts, a pad of 2 gives 1).  FP64 keeps a pad of 1.
int fused_q_stride(int N, int rs, int P, int G, int esz) {
    const int base = N * rs;
    if (esz != 4 || G >= 32) return base + 1;
    const int C = (P + G - 1) / G;
    int best = base + 1, best_cost = -1;
    for (int d = 1; d <= 32; ++d) {
        const int qs = base + d;
        int cost = 0;
        for (int ii = 0; ii < C; ++ii) {
            int cnt[32] = {};
            int worst = 0;
            for (int t = 0; t < 32; ++t) {
                const int p = (t % G) * C + ii;
                if (p >= P) continue;
                const int w = (t / G) * qs + p + (p >> 5);
                worst = std::max(worst, ++cnt[w & 31]);
            }
            cost += worst;
        }
        if (best_cost < 0 || cost < best_cost) { best_cost = cost; best = qs; }
    }
    return best;
}

int run_fused(const pbr_model* model, int qmode, const void* q_in, int64_t X, uint64_t seed,
              uint64_t offset, const pbr_outputs* out, void* stream) {
    using namespace pbr;
    if (!model || !out || X < 0) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const pbr_model& m = *model;
    const int chk = check_model(m, qmode, q_in, out);
    if (chk != PBR_OK) return chk;
    const bool team = m.variant >= 2 || (m.variant == 0 && m.A > 4);
    if (team) return run_team(m, qmode, q_in, X, seed, offset, out, static_cast<cudaStream_t>(stream));
    if (m.A > 4) return PBR_ERR_UNSUPPORTED;

    FusedArgs a;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    a.q_in = q_in;
    a.X = X;
    a.out = *out;
    a.key0 = static_cast<uint32_t>(seed);
    a.key1 = static_cast<uint32_t>(seed >> 32);
    a.offset = offset;
    a.rs = row_stride(m.P);
    // threads per sample: enough that each owns <= kMaxChunk beads, more (up to a warp) when
    // the per-CTA shared memory of S = kThreads / G samples would not fit
    const int esz = m.precision == 32 ? 4 : 8;
    a.G = std::min(32, pow2ceil((m.P + kMaxChunk - 1) / kMaxChunk));
    while (true) {
        a.S = kThreads / a.G;
        a.qstride = fused_q_stride(m.N, a.rs, m.P, a.G, esz);
        // the tensor-core quadratic where it applies and its tables fit, else the pair loop
        const SmemPlan pt(m.A, m.K, qmode, esz, m.N, m.P, a.S, a.qstride, 1);
        const SmemPlan p0(m.A, m.K, qmode, esz, m.N, m.P, a.S, a.qstride, 0);
        if (pt.total_bytes <= kMaxSmem) { a.tcq = pt.tcq_k > 0 ? 1 : 0; break; }
        if (p0.total_bytes <= kMaxSmem) { a.tcq = 0; break; }
        if (a.G == 32) return PBR_ERR_UNSUPPORTED;
        a.G *= 2;
    }
    a.logG = ilog2(a.G);
    a.C = (m.P + a.G - 1) / a.G;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    switch (m.A) {
        case 1: return launch_fused<1>(m.K, qmode, m.precision, a, st);
        case 2: return launch_fused<2>(m.K, qmode, m.precision, a, st);
        case 3: return launch_fused<3>(m.K, qmode, m.precision, a, st);
        case 4: return launch_fused<4>(m.K, qmode, m.precision, a, st);
        default: return PBR_ERR_UNSUPPORTED;
    }
}

}  // namespace

extern "C" {

int pbr_sample_eval(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X,
                    const pbr_outputs* out, void* stream) {
    return run_fused(model, pbr::kSample, nullptr, X, seed, offset, out, stream);
}

int pbr_eval_q(const pbr_model* model, const double* q, int64_t X, const pbr_outputs* out,
               void* stream) {
    return run_fused(model, pbr::kQ64, q, X, 0, 0, out, stream);
}

int pbr_eval_q_f32(const pbr_model* model, const float* q, int64_t X, const pbr_outputs* out,
                   void* stream) {
    if (model && model->precision != 32) return PBR_ERR_ARG;
    return run_fused(model, pbr::kQ32, q, X, 0, 0, out, stream);
}

int pbr_sample_q(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X,
                 float* q_out, int32_t* src_out, void* stream) {
    using namespace pbr;
    if (!model || !q_out || X < 0) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const pbr_model& m = *model;
    if (m.N < 1 || m.N > PBR_MAX_N || m.P < 3 || m.P > PBR_MAX_P) return PBR_ERR_ARG;
    if (m.A_rho < 1 || m.A_rho > PBR_MAX_A_RHO || !m.ring_chol || !m.src_cdf || !m.rho_d) return PBR_ERR_ARG;
    if (m.precision != 32 && m.precision != 64) return PBR_ERR_ARG;
    FusedArgs a;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    a.X = X;
    a.out.q_out = q_out;
    a.out.src_out = src_out;
    a.key0 = static_cast<uint32_t>(seed);
    a.key1 = static_cast<uint32_t>(seed >> 32);
    a.offset = offset;
    a.rs = row_stride(m.P);
    a.qstride = m.N * a.rs + 1;
    const size_t esz = m.precision == 32 ? sizeof(float) : sizeof(double);
    a.G = std::min(32, pow2ceil((m.P + kMaxChunk - 1) / kMaxChunk));
    int bytes = 0;
    while (true) {
        a.S = kThreads / a.G;
        bytes = static_cast<int>(a.S * a.qstride * esz);
        if (bytes <= kMaxSmem || a.G == 32) break;
        a.G *= 2;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (bytes > kMaxSmem || m.precision == 32) {
        // FP32: the row-streaming form (one mode of 32 samples per warp, lane = sample), the same
        // bits as the staged form and measured 1.8-4.1x faster on GB300 (A = 3-8, N = 6-20,
        // P = 16-256: more warps per SM hide the chains' latency); FP64 samples too large to
        // stage have no form
        if (m.precision != 32) return PBR_ERR_UNSUPPORTED;
        int dev = 0, sms = 0;
        PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
        PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int64_t warps = (X + 31) / 32 * m.N;
        const int64_t blocks = (warps + kRowsWarps - 1) / kRowsWarps;
        const int grid = static_cast<int>(std::min<int64_t>(blocks, static_cast<int64_t>(sms) * 8));
        sample_q_rows_kernel<float><<<grid, kRowsWarps * 32, 0, st>>>(a);
        return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
    }
    a.logG = ilog2(a.G);
    a.C = (m.P + a.G - 1) / a.G;
    auto go = [&](auto kern) -> int {
        if (bytes > 48 * 1024 &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
            return PBR_ERR_UNSUPPORTED;
        int dev = 0, sms = 0, occ = 0;
        PBR_CUDA_CHECK_RET(cudaGetDevice(&dev));
        PBR_CUDA_CHECK_RET(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PBR_CUDA_CHECK_RET(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreads, bytes));
        if (occ < 1) return PBR_ERR_UNSUPPORTED;
        const int64_t need = (X + a.S - 1) / a.S;
        const int grid = static_cast<int>(std::min<int64_t>(need, static_cast<int64_t>(occ) * sms));
        kern<<<grid, kThreads, bytes, st>>>(a);
        return cudaGetLastError() == cudaSuccess ? PBR_OK : PBR_ERR_CUDA;
    };
    if (m.precision == 32) return go(sample_q_kernel<float>);
    return go(sample_q_kernel<double>);
}

// ---- batched multi-model launch ------------------------------------------------------------
namespace {
constexpr int kBatchMaxGroups = 32;
// chunked: the group's models run as one register-chunk launch each instead of the batched
// row-team launch (up to 4 surfaces the chunk form is 2.2-3x faster per sample; the launches
// are short enough to sit in the same CUDA graph)
struct BatchGroup {
    int32_t A, K, n_items, smem_bytes, chunked, tcq;
    int64_t first_item, total_tiles;
};
struct BatchHeader {
    int32_t n_groups, n_items, grid_cap, pad;
    BatchGroup groups[kBatchMaxGroups];
};
}  // namespace

int64_t pbr_batch_blob_bytes(int32_t n_models) {
    return static_cast<int64_t>(sizeof(BatchHeader)) + static_cast<int64_t>(n_models) * sizeof(pbr::TeamBatchItem);
}

int pbr_batch_pack(const pbr_model* models, const uint64_t* seeds, const uint64_t* offsets, const int64_t* X,
                   const pbr_outputs* outs, int32_t n_models, const int32_t* smem_budgets, int32_t grid_cap,
                   void* host_blob) {
    using namespace pbr;
    if (!models || !seeds || !offsets || !X || !outs || !host_blob || n_models < 1) return PBR_ERR_ARG;
    // per surface count: < 0 the register-chunk launches (up to 4 surfaces), 0 the whole shared
    // memory, > 0 a shared-memory budget for the row-team tiles; no table: chunks up to 4
    // surfaces, the whole shared memory beyond
    auto budget_of = [&](int A) { return smem_budgets ? smem_budgets[A] : (A <= 4 ? -1 : 0); };
    auto* hdr = static_cast<BatchHeader*>(host_blob);
    auto* items = reinterpret_cast<TeamBatchItem*>(hdr + 1);
    std::memset(hdr, 0, sizeof(BatchHeader));
    hdr->grid_cap = grid_cap;
    int n = 0;
    // group by (A, K) in increasing A; at 5-6 surfaces by whether two tiles fit an SM (those
    // models run the two-block build); of the one-block models, those whose bead records take
    // the tensor-core quadratic (5-8 surfaces, from 16 modes, tables within the budget) form
    // their own group (cls 2); within a group keep the caller's order
    for (int A = 1; A <= PBR_MAX_A; ++A)
        for (int K = 0; K <= 4; K += 4)
        for (int cls = 0; cls < 3; ++cls) {
            const int first = n;
            int64_t tiles = 0;
            int smem = 0;
            const int ba = budget_of(A);
            const int budget = (ba > 0 && ba < kMaxSmem) ? ba : kMaxSmem;
            bool chunked = A <= 4 && ba < 0;
            for (int i = 0; i < n_models; ++i) {
                const pbr_model& m = models[i];
                if (m.A != A || m.K != K) continue;
                if (m.precision != 32 || m.A_rho < m.A || m.n_fill_rho != m.A || m.N < 1 ||
                    m.N > PBR_MAX_N || m.P < 3 || m.P > PBR_MAX_P || X[i] < 0 || !outs[i].s_rho || !outs[i].s_g ||
                    (K > 0 && (!outs[i].s_gp || !outs[i].s_gm)) || !m.ring_chol || !m.src_cdf)
                    return PBR_ERR_ARG;
                TeamArgs a;
                int rc = make_team_args(m, kSample, nullptr, X[i], seeds[i], offsets[i], &outs[i], budget, &a);
                // a model whose one-sample tile does not fit the budget takes the full shared
                // memory instead of vetoing the budget for the whole batch
                if (rc == PBR_ERR_UNSUPPORTED && budget < kMaxSmem)
                    rc = make_team_args(m, kSample, nullptr, X[i], seeds[i], offsets[i], &outs[i], kMaxSmem, &a);
                if (rc != PBR_OK) return rc;
                const bool two = (A == 5 || A == 6) && team_smem(a, kSample) <= kTeamTwoBlockSmem;
                if (!two) choose_team_tcq(a, kSample, budget);
                const int c = two ? 0 : (a.tcq ? 2 : 1);
                if (c != cls) continue;
                TeamBatchItem& it = items[n];
                it.a = a;
                it.tile_begin = tiles;
                tiles += (X[i] + it.a.S - 1) / it.a.S;
                smem = std::max(smem, team_smem(it.a, kSample));
                chunked = chunked && (m.variant == 0 || m.variant == 1);   // a model asking for teams keeps them
                ++n;
            }
            if (n > first) {
                if (hdr->n_groups >= kBatchMaxGroups) return PBR_ERR_UNSUPPORTED;
                BatchGroup& g = hdr->groups[hdr->n_groups++];
                g.A = A; g.K = K; g.n_items = n - first; g.smem_bytes = smem;
                g.chunked = chunked ? 1 : 0;
                g.tcq = cls == 2 ? 1 : 0;
                g.first_item = first; g.total_tiles = tiles;
            }
        }
    if (n != n_models) return PBR_ERR_ARG;
    hdr->n_items = n;
    return PBR_OK;
}

int pbr_sample_eval_batch(const void* host_blob, const void* device_blob, void* stream) {
    using namespace pbr;
    if (!host_blob || !device_blob) return PBR_ERR_ARG;
    const auto* hdr = static_cast<const BatchHeader*>(host_blob);
    const auto* items = reinterpret_cast<const TeamBatchItem*>(
        static_cast<const char*>(device_blob) + sizeof(BatchHeader));
    const auto* hitems = reinterpret_cast<const TeamBatchItem*>(hdr + 1);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int gi = 0; gi < hdr->n_groups; ++gi) {
        const BatchGroup& g = hdr->groups[gi];
        if (g.total_tiles == 0) continue;
        if (g.chunked) {
            // one register-chunk launch per model, from the host copy of its arguments
            for (int64_t i = g.first_item; i < g.first_item + g.n_items; ++i) {
                const TeamArgs& a = hitems[i].a;
                const uint64_t seed = static_cast<uint64_t>(a.key0) | (static_cast<uint64_t>(a.key1) << 32);
                const int rc = run_fused(&a.m, kSample, nullptr, a.X, seed, a.offset, &a.out, stream);
                if (rc != PBR_OK) return rc;
            }
            continue;
        }
        const TeamBatchItem* gitems = items + g.first_item;
        int rc = PBR_ERR_UNSUPPORTED;
        switch (g.A) {
            case 1: rc = launch_team_batch<1>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 2: rc = launch_team_batch<2>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 3: rc = launch_team_batch<3>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 4: rc = launch_team_batch<4>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 5: rc = launch_team_batch<5>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 6: rc = launch_team_batch<6>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 7: rc = launch_team_batch<7>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            case 8: rc = launch_team_batch<8>(g.K, gitems, g.n_items, g.total_tiles, g.smem_bytes, hdr->grid_cap, g.tcq, st); break;
            default: break;
        }
        if (rc != PBR_OK) return rc;
    }
    return PBR_OK;
}

int32_t pbr_batch_groups(const void* host_blob) {
    return host_blob ? static_cast<const BatchHeader*>(host_blob)->n_groups : 0;
}

const char* pbr_version(void) { return "pibronic_gb300 0.1 sm_103a"; }

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Tensor-core form: per chunk of samples, (1) the sampler writes q, (2) the tcgen05 contraction
// writes the quadratic coupling part of V for every (sample, bead) row, (3) the row-team kernel
// evaluates the chunk from q and that V.  The chunk is sized by the caller's scratch; about
// 64 MB of q and V per chunk keeps both resident in L2 between the three launches.
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int64_t kScratchAlign = 256;

int64_t align_bytes(int64_t n) { return (n + kScratchAlign - 1) / kScratchAlign * kScratchAlign; }

int64_t tc_fixed_bytes(const pbr_model& m) {
    return align_bytes(pbr::tc_packed_floats(m.N, m.A) * 4) + kScratchAlign;
}

// The wide form's tile: up to 16 teams per sample, windows of up to 8 beads per team.
pbr::WideArgs make_wide_args(const pbr_model& m, const float* q, const float* vq, int ld, int64_t X,
                             const pbr_outputs* out) {
    using namespace pbr;
    WideArgs a;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    a.q = q;
    a.vq = vq;
    a.vq_ld = ld;
    a.X = X;
    if (out) a.out = *out;
    a.G = std::min(kWideTeams, m.P);
    a.C = (m.P + a.G - 1) / a.G;
    a.W = std::min(a.C, 8);
    return a;
}

int run_wide(const pbr_model& m, const float* q, const float* vq, int ld, int64_t X, const pbr_outputs* out,
             cudaStream_t st) {
    using namespace pbr;
    const WideArgs a = make_wide_args(m, q, vq, ld, X, out);
    if (m.A <= 12) return launch_wide<12>(m.K, a, st);
    return launch_wide<16>(m.K, a, st);
}

// samples the wide kernel evaluates in one wave (one per resident block); 0 when it cannot run
int64_t wide_wave(const pbr_model& m, int ld) {
    using namespace pbr;
    const WideArgs a = make_wide_args(m, nullptr, nullptr, ld, 1, nullptr);
    return m.A <= 12 ? wide_resident<12>(m.K, a) : wide_resident<16>(m.K, a);
}

int64_t tc_sample_bytes(const pbr_model& m) {
    return static_cast<int64_t>(m.N) * m.P * 4 + static_cast<int64_t>(m.P) * pbr::tc_quadratic_cols(m.A) * 4;
}

}  // namespace

extern "C" {

int64_t pbr_sample_eval_tc_scratch(const pbr_model* model, int64_t chunk) {
    if (!model || chunk < 1 || model->A < 1 || model->A > PBR_MAX_A_WIDE || model->N < 1 || model->N > PBR_MAX_N ||
        model->P < 3 || model->P > PBR_MAX_P)
        return -1;
    return tc_fixed_bytes(*model) + 2 * kScratchAlign + chunk * tc_sample_bytes(*model);
}

}  // extern "C"

namespace {

// the chunked tensor-core pipeline; q_in == nullptr: draw q with the sampler
int run_tc(const pbr_model* model, const float* q_in, uint64_t seed, uint64_t offset, int64_t X,
           const pbr_outputs* out, void* scratch, int64_t scratch_bytes, void* stream) {
    using namespace pbr;
    if (!model || !out || X < 0 || !scratch) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const pbr_model& m = *model;
    const int chk = q_in ? check_model(m, kQ32, q_in, out, PBR_MAX_A_WIDE)
                         : check_model(m, kSample, nullptr, out, PBR_MAX_A_WIDE);
    if (chk != PBR_OK) return chk;
    if (m.precision != 32) return PBR_ERR_UNSUPPORTED;        // FP16 split: the FP32 form only
    const bool wide = m.A > PBR_MAX_A;
    if (reinterpret_cast<uintptr_t>(scratch) % kScratchAlign) return PBR_ERR_ARG;
    const int64_t per = tc_sample_bytes(m);
    int64_t chunk = (scratch_bytes - tc_fixed_bytes(m) - 2 * kScratchAlign) / per;
    if (chunk < 1) return PBR_ERR_CAPACITY;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int A2P = tc_quadratic_cols(m.A);
    if (wide && chunk < X) {
        // the wide kernel takes one sample per block: a chunk of whole waves leaves no block idle
        // while others finish a last sample (455 samples on 304 resident blocks ran as 2 waves of
        // which the second was half empty)
        const int64_t wave = wide_wave(m, A2P);
        if (wave > 0 && chunk >= wave) chunk = chunk / wave * wave;
    }
    unsigned char* base = static_cast<unsigned char*>(scratch);
    void* bpack = base;
    float* qbuf = reinterpret_cast<float*>(base + tc_fixed_bytes(m));
    float* vq = reinterpret_cast<float*>(base + tc_fixed_bytes(m) +
                                         align_bytes(chunk * static_cast<int64_t>(m.N) * m.P * 4));
    int rc = tc_pack_launch(m.vib_qq, m.vib_l, m.vib_e, m.precision, m.N, m.A, bpack, st);
    if (rc != PBR_OK) return rc;
    const int K1 = m.K + 1;
    const int64_t NP = static_cast<int64_t>(m.N) * m.P;
    for (int64_t c0 = 0; c0 < X; c0 += chunk) {
        const int64_t n = std::min(chunk, X - c0);
        const float* qc;
        if (q_in) {
            qc = q_in + c0 * NP;
        } else {
            float* qs = out->q_out ? out->q_out + c0 * NP : qbuf;
            rc = pbr_sample_q(model, seed, offset + static_cast<uint64_t>(c0), n, qs,
                              out->src_out ? out->src_out + c0 : nullptr, stream);
            if (rc != PBR_OK) return rc;
            qc = qs;
        }
        rc = tc_quadratic_launch(qc, n, m.N, m.P, m.A, bpack, vq, out->status, st);
        if (rc != PBR_OK) return rc;
        pbr_outputs oc = *out;
        oc.s_rho = out->s_rho + c0;
        oc.s_g = out->s_g + c0;
        oc.s_gp = out->s_gp ? out->s_gp + c0 : nullptr;
        oc.s_gm = out->s_gm ? out->s_gm + c0 : nullptr;
        oc.g_coef = out->g_coef ? out->g_coef + c0 * K1 : nullptr;
        oc.log_scale = out->log_scale ? out->log_scale + c0 : nullptr;
        oc.q_out = nullptr;
        oc.src_out = nullptr;
        rc = wide ? run_wide(m, qc, vq, A2P, n, &oc, st) : run_team(m, kQ32V, qc, n, 0, 0, &oc, st, vq, A2P);
        if (rc != PBR_OK) return rc;
    }
    return PBR_OK;
}

}  // namespace

extern "C" {

int pbr_sample_eval_tc(const pbr_model* model, uint64_t seed, uint64_t offset, int64_t X, const pbr_outputs* out,
                       void* scratch, int64_t scratch_bytes, void* stream) {
    return run_tc(model, nullptr, seed, offset, X, out, scratch, scratch_bytes, stream);
}

int pbr_eval_q_tc(const pbr_model* model, const float* q, int64_t X, const pbr_outputs* out, void* scratch,
                  int64_t scratch_bytes, void* stream) {
    if (!q) return PBR_ERR_ARG;
    return run_tc(model, q, 0, 0, X, out, scratch, scratch_bytes, stream);
}

}  // extern "C"
