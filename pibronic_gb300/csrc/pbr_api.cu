// pbr_api.cu -- extern "C" entry points of the fused path (declared in include/pibronic_gb300.h).
#include <algorithm>
#include <cstring>

#include "pbr_team.cuh"

namespace pbr {
template <int A> int launch_fused(int, int, int, const FusedArgs&, cudaStream_t);
template <int A> int launch_team(int, int, int, const TeamArgs&, cudaStream_t);
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

int run_team(const pbr_model& m, int qmode, const void* q_in, int64_t X, uint64_t seed,
             uint64_t offset, const pbr_outputs* out, cudaStream_t st) {
    using namespace pbr;
    TeamArgs a;
    std::memset(&a, 0, sizeof(a));
    a.m = m;
    a.q_in = q_in;
    a.X = X;
    a.out = *out;
    a.key0 = static_cast<uint32_t>(seed);
    a.key1 = static_cast<uint32_t>(seed >> 32);
    a.offset = offset;
    a.rs = row_stride(m.P);
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
        if (plan.total_bytes <= kMaxSmem) break;
        if (a.S == 1) return PBR_ERR_UNSUPPORTED;
        a.S = std::max(1, a.S / 2);
    }
    a.C = (m.P + a.G - 1) / a.G;
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

int run_fused(const pbr_model* model, int qmode, const void* q_in, int64_t X, uint64_t seed,
              uint64_t offset, const pbr_outputs* out, void* stream) {
    using namespace pbr;
    if (!model || !out || X < 0) return PBR_ERR_ARG;
    if (X == 0) return PBR_OK;
    const pbr_model& m = *model;
    if (m.A < 1 || m.A > PBR_MAX_A) return PBR_ERR_UNSUPPORTED;
    if (m.variant < 0 || m.variant > 2) return PBR_ERR_ARG;
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
    const bool team = m.variant == 2 || (m.variant == 0 && m.A > 4);
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
    a.qstride = m.N * a.rs + 1;
    // threads per sample: enough that each owns <= kMaxChunk beads, more (up to a warp) when
    // the per-CTA shared memory of S = kThreads / G samples would not fit
    const int esz = m.precision == 32 ? 4 : 8;
    a.G = std::min(32, pow2ceil((m.P + kMaxChunk - 1) / kMaxChunk));
    while (true) {
        a.S = kThreads / a.G;
        const SmemPlan plan(m.A, m.K, qmode, esz, m.N, m.P, a.S, a.qstride);
        if (plan.total_bytes <= kMaxSmem || a.G == 32) {
            if (plan.total_bytes > kMaxSmem) return PBR_ERR_UNSUPPORTED;
            break;
        }
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
    if (bytes > kMaxSmem) return PBR_ERR_UNSUPPORTED;
    a.logG = ilog2(a.G);
    a.C = (m.P + a.G - 1) / a.G;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
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

const char* pbr_version(void) { return "pibronic_gb300 0.1 sm_103a"; }

}  // extern "C"
