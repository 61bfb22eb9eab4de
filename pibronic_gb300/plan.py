"""Host FP64 precompute of the model constants and their device tables (the pbr_model struct).

This is the work of BoxData.preprocess / ModelVibronic(PM).precompute / ModelSampling.precompute
(pimc.py:59-89, 172-424, 647-738), restated for the fused kernel:

* The O-matrix exponent is carried as a truncated Taylor series in the beta step h,
  phi_pa(beta + h) = sum_k phi_pa,k h^k (order K = 4 on the plus/minus path), so g(beta +- db)
  (pimc.py:1442-1449) come out of one ring product as sum_k Tr N_k (+-db)^k.  Only the harmonic
  O matrices depend on h; M always uses the central tau, as in the reference.
* The coefficients of csch(w (beta+h)/P), tanh(w (beta+h)/(2P)) and ln prefactor(beta+h) are
  built here with truncated-power-series arithmetic in FP64.
"""
from __future__ import annotations

import math

import numpy as np

from .constants import beta as beta_of

F64 = np.float64


# ---------------------------------------------------------------------------------------------
# truncated power series (coefficient arrays along the last axis)
# ---------------------------------------------------------------------------------------------
def tps_sinh_cosh(x0, slope, K):
    """Series of sinh and cosh of x0 + slope*h: d^k/dh^k alternates between sinh and cosh."""
    x0 = np.asarray(x0, dtype=F64)
    slope = np.asarray(slope, dtype=F64)
    sh, ch = np.sinh(x0), np.cosh(x0)
    S = np.empty(x0.shape + (K + 1,))
    Cc = np.empty(x0.shape + (K + 1,))
    for k in range(K + 1):
        f = slope ** k / math.factorial(k)
        S[..., k] = f * (sh if k % 2 == 0 else ch)
        Cc[..., k] = f * (ch if k % 2 == 0 else sh)
    return S, Cc


def tps_recip(a):
    K = a.shape[-1] - 1
    r = np.zeros_like(a)
    r[..., 0] = 1.0 / a[..., 0]
    for k in range(1, K + 1):
        acc = np.zeros(a.shape[:-1])
        for i in range(1, k + 1):
            acc += a[..., i] * r[..., k - i]
        r[..., k] = -acc / a[..., 0]
    return r


def tps_mul(a, b):
    K = a.shape[-1] - 1
    c = np.zeros(np.broadcast(a[..., 0], b[..., 0]).shape + (K + 1,))
    for k in range(K + 1):
        for i in range(k + 1):
            c[..., k] += a[..., i] * b[..., k - i]
    return c


def tps_log(a):
    K = a.shape[-1] - 1
    lg = np.zeros_like(a)
    lg[..., 0] = np.log(a[..., 0])
    for k in range(1, K + 1):
        acc = a[..., k] * k
        for i in range(1, k):
            acc = acc - i * lg[..., i] * a[..., k - i]
        lg[..., k] = acc / (k * a[..., 0])
    return lg


def harmonic_series(omega, beta, P, K):
    """Taylor coefficients in h of csch(w(beta+h)/P), tanh(w(beta+h)/(2P)) and ln sinh(w(beta+h)/P).
    Shapes (N, K+1)."""
    omega = np.asarray(omega, dtype=F64)
    s1, c1 = tps_sinh_cosh(omega * beta / P, omega / P, K)
    s2, c2 = tps_sinh_cosh(omega * beta / (2 * P), omega / (2 * P), K)
    return tps_recip(s1), tps_mul(s2, tps_recip(c2)), tps_log(s1)


def prefactor_log_series(tilde_energy, omega, beta, P, K):
    """ln[exp(-tau Etilde_a) prod_j csch(tau w_j)^(1/2)] at tau = (beta+h)/P, shape (A, K+1)
    (pimc.py:74-81)."""
    _, _, lsinh = harmonic_series(omega, beta, P, K)
    out = np.zeros((len(tilde_energy), K + 1))
    out[:, 0] = -beta / P * tilde_energy
    if K >= 1:
        out[:, 1] = -tilde_energy / P
    out -= 0.5 * lsinh.sum(axis=0)[None, :]
    return out


# ---------------------------------------------------------------------------------------------
# ring normal modes
# ---------------------------------------------------------------------------------------------
def ring_mode_eigenvalues(P):
    """Eigenvalues of the ring adjacency C (circulant [0,1,0..0,1], pimc.py:684-689) in the real
    Fourier order the sampler uses: slot 0 constant, slots 2k-1, 2k the cos/sin pair of
    frequency k, slot P-1 the alternating mode when P is even."""
    lam = np.empty(P)
    lam[0] = 2.0
    for k in range(1, (P - 1) // 2 + 1):
        lam[2 * k - 1] = lam[2 * k] = 2.0 * math.cos(2.0 * math.pi * k / P)
    if P % 2 == 0:
        lam[P - 1] = -2.0
    return lam


def ring_mode_basis(P):
    """The orthonormal basis B[p, s] matching ring_mode_eigenvalues (q_p = sum_s B_ps cc_s)."""
    p = np.arange(P)
    B = np.empty((P, P))
    B[:, 0] = 1.0 / math.sqrt(P)
    for k in range(1, (P - 1) // 2 + 1):
        B[:, 2 * k - 1] = math.sqrt(2.0 / P) * np.cos(2 * math.pi * k * p / P)
        B[:, 2 * k] = math.sqrt(2.0 / P) * np.sin(2 * math.pi * k * p / P)
    if P % 2 == 0:
        B[:, P - 1] = (-1.0) ** p / math.sqrt(P)
    return B


def ring_precision_factor(omega, tau, P):
    """Back-substitution coefficients of the bead-space precision of rho for each mode,
    Lambda_j = 2 coth(tau w_j) I - csch(tau w_j) C (pimc.py:402-404 in the normal-mode basis).
    Lambda_j is cyclic tridiagonal, so its Cholesky factor L is bidiagonal plus a dense last row,
    and x = L^-T z solves as x_p = a_p (z_p - b_p x_{p+1} - c_p x_{P-1}).  Returns (3, N, P):
    a = 1/L_pp, b_p = L_{p+1,p} (p <= P-3) and L_{P-1,P-2} (p = P-2), c_p = L_{P-1,p} (p <= P-3)."""
    omega = np.asarray(omega, dtype=F64)
    N = omega.shape[0]
    C = np.zeros((P, P))
    for p in range(P):
        C[p, (p + 1) % P] = C[p, (p - 1) % P] = 1.0
    out = np.zeros((3, N, P))
    for j in range(N):
        lam = 2.0 / np.tanh(tau * omega[j]) * np.eye(P) - C / np.sinh(tau * omega[j])
        L = np.linalg.cholesky(lam)
        out[0, j] = 1.0 / np.diag(L)
        out[1, j, :P - 2] = np.array([L[p + 1, p] for p in range(P - 2)])
        out[1, j, P - 2] = L[P - 1, P - 2]
        out[2, j, :P - 2] = L[P - 1, :P - 2]
    return out


def pair_index(b, c):
    return b * (b + 1) // 2 + c


# ---------------------------------------------------------------------------------------------
# prepared models
# ---------------------------------------------------------------------------------------------
class PreparedModels:
    """Everything the device tables are built from (FP64, host)."""

    def __init__(self, vib, rho, P, temperature=None, beta=None, delta_beta=None, K=None):
        from .vibronic_io import VMK
        self.beta = beta if beta is not None else beta_of(temperature)
        self.P = P
        self.tau = self.beta / P
        self.delta_beta = 0.0 if delta_beta is None else float(delta_beta)
        self.K = (4 if delta_beta is not None else 0) if K is None else K
        A, N = int(vib[VMK.A]), int(vib[VMK.N])
        Ar = int(rho[VMK.A])
        assert int(rho[VMK.N]) == N, "sampling and coupled models must have the same modes"
        self.A, self.N, self.A_rho = A, N, Ar
        assert P >= 3, "circulant matrix requires 3 or more beads"
        # reference fills min(A, A_rho) rho surfaces and fails when A_rho < A (pimc.py:1110)
        assert Ar >= A, "the sampling model needs at least as many surfaces as the coupled model"
        self.n_fill_rho = A
        w = np.asarray(vib[VMK.w], dtype=F64)
        E = np.array(vib[VMK.E], dtype=F64)
        L = np.array(vib[VMK.G1], dtype=F64)
        Q = np.array(vib[VMK.G2], dtype=F64)
        lin_diag = np.array([L[:, a, a] for a in range(A)])              # (A,N)
        self.vib_delta = -0.5 * (lin_diag ** 2 / w[None, :]).sum(axis=1)  # pimc.py:176
        self.vib_tilde = np.diag(E) + self.vib_delta                      # pimc.py:75-76
        self.vib_shift = -lin_diag / w[None, :]                            # pimc.py:212
        for a in range(A):                                                 # pimc.py:214-217
            L[:, a, a] = 0.0
            E[a, a] = 0.0
        # V(q) must be symmetric in the surfaces (pimc.py:1169)
        assert np.allclose(E, E.T) and np.allclose(L, L.transpose(0, 2, 1)) \
            and np.allclose(Q, Q.transpose(0, 1, 3, 2)), "coupling terms are not symmetric in surfaces"
        self.vib_omega, self.vib_E, self.vib_L, self.vib_Q = w, E, L, Q
        wr = np.asarray(rho[VMK.w], dtype=F64)
        Lr = np.asarray(rho[VMK.G1], dtype=F64)                            # (N, A_rho)
        self.rho_delta = -0.5 * (Lr ** 2 / wr[:, None]).sum(axis=0)       # pimc.py:338
        Er = np.asarray(rho[VMK.E], dtype=F64)
        weight = np.exp(-self.beta * (Er + self.rho_delta))               # pimc.py:343
        weight /= np.prod(np.sinh(self.beta * wr / 2.0))                  # pimc.py:347
        self.state_weight = weight / weight.sum()                         # pimc.py:350
        self.rho_tilde = Er + self.rho_delta
        self.rho_shift = (-Lr / wr[:, None]).T.copy()                     # pimc.py:376
        self.rho_omega = wr

    # -- host constants ----------------------------------------------------------------------
    def tables(self):
        """FP64 numpy tables keyed like the pbr_model fields, plus log_c0."""
        A, N, P, K, Ar = self.A, self.N, self.P, self.K, self.A_rho
        csch_s, tanh_s, _ = harmonic_series(self.vib_omega, self.beta, P, K)
        vib_c = prefactor_log_series(self.vib_tilde, self.vib_omega, self.beta, P, K)  # (A,K+1)
        rcsch, rtanh, _ = harmonic_series(self.rho_omega, self.beta, P, 0)
        rho_c = prefactor_log_series(self.rho_tilde, self.rho_omega, self.beta, P, 0)[:, 0]
        log_c0 = float(max(vib_c[:, 0].max(), rho_c[:A].max()))
        vib_c[:, 0] -= log_c0
        rho_c = rho_c - log_c0
        A2, N2 = A * (A + 1) // 2, N * (N + 1) // 2
        e = np.array([self.vib_E[b, c] for b in range(A) for c in range(b + 1)])
        lt = np.array([[self.vib_L[j, b, c] for b in range(A) for c in range(b + 1)] for j in range(N)])
        Q = self.vib_Q
        qq = np.empty((N2, A2))
        for d in range(N):
            for e_ in range(d + 1):
                row = pair_index(d, e_)
                for b in range(A):
                    for c in range(b + 1):
                        if d == e_:
                            qq[row, pair_index(b, c)] = 0.5 * Q[d, d, b, c]
                        else:
                            qq[row, pair_index(b, c)] = 0.5 * (Q[d, e_, b, c] + Q[e_, d, b, c])
        # bead-major [3][P][N]: the threads that run different modes at one bead read neighbours
        ring_chol = np.ascontiguousarray(ring_precision_factor(self.rho_omega, self.tau, P).transpose(0, 2, 1))
        return {
            "vib_cs": 0.5 * csch_s.T.copy(), "vib_th": 0.5 * tanh_s.T.copy(), "vib_c": vib_c.T.copy(),
            "vib_d": self.vib_shift.copy(), "vib_e": e, "vib_l": lt.reshape(N, A2), "vib_qq": qq,
            "rho_cs": 0.5 * rcsch[:, 0], "rho_th": 0.5 * rtanh[:, 0], "rho_c": rho_c,
            "rho_d": self.rho_shift.copy(), "ring_chol": ring_chol,
            "src_cdf": np.cumsum(self.state_weight), "log_c0": log_c0,
        }


class DevicePlan:
    """The device-resident tables of one PreparedModels and the pbr_model struct pointing at them."""

    FIELDS = ("vib_cs", "vib_th", "vib_c", "vib_d", "vib_e", "vib_l", "vib_qq", "rho_cs", "rho_th",
              "rho_c", "rho_d", "ring_chol", "src_cdf")

    #: fused-kernel forms (pbr_model.variant): register-resident chunks (A <= 4), bead-parallel
    #: records + row teams (A <= 8), or row teams fed by the tensor-core quadratic contraction
    #: (pbr_sample_eval_tc, precision 32); 0 lets the library choose
    VARIANT_AUTO, VARIANT_CHUNK, VARIANT_TEAM, VARIANT_TC = 0, 1, 2, 3

    #: auto choice of the tensor-core form (measured on GB300, samples/s of both forms): from 5
    #: surfaces on, when the quadratic coupling table of the shared-memory forms (npair(N) x
    #: align4(npair(A)) FP32 values) exceeds this many bytes; always beyond 8 surfaces; and for
    #: any shape the shared-memory forms cannot hold (evaluate_device retries on the tensor-core
    #: form when they report unsupported sizes).  Up to 4 surfaces the row-team / chunk forms win
    #: at every N <= 64.
    TC_TABLE_BYTES = 64 * 1024
    TC_MIN_A = 5
    #: q and V bytes per chunk of the tensor-core form (L2-resident between its launches)
    TC_CHUNK_BYTES = 64 << 20

    def __init__(self, prep, precision=32, device=None, variant=0):
        from . import _native
        torch = _native.require_cuda()
        assert precision in (32, 64)
        assert 1 <= prep.A <= 16, "the kernels support 1 to 16 coupled surfaces"
        assert prep.A <= 8 or (precision == 32 and variant in (self.VARIANT_AUTO, self.VARIANT_TC)), \
            "9 to 16 surfaces run on the tensor-core form only (precision 32)"
        self.prep, self.precision = prep, precision
        tabs = prep.tables()
        dt = torch.float32 if precision == 32 else torch.float64
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.tensors = {k: torch.as_tensor(np.ascontiguousarray(tabs[k]).ravel(), dtype=dt).to(dev)
                        for k in self.FIELDS}
        m = _native.PbrModel()
        m.A, m.A_rho, m.n_fill_rho, m.N, m.P, m.K = prep.A, prep.A_rho, prep.n_fill_rho, prep.N, prep.P, prep.K
        m.precision = precision
        m.variant = variant
        m.tau, m.delta_beta, m.log_c0 = prep.tau, prep.delta_beta, tabs["log_c0"]
        for k in self.FIELDS:
            setattr(m, k, self.tensors[k].data_ptr())
        self.struct = m
        self.log_c0 = tabs["log_c0"]
        self.variant = variant
        n2, a2p = prep.N * (prep.N + 1) // 2, (prep.A * (prep.A + 1) // 2 + 3) // 4 * 4
        self.use_tc = precision == 32 and (variant == self.VARIANT_TC or prep.A > 8 or (
            variant == self.VARIANT_AUTO and prep.A >= self.TC_MIN_A and n2 * a2p * 4 > self.TC_TABLE_BYTES))
        self._tc_scratch = None

    def tc_scratch(self):
        """Device scratch of the tensor-core form (allocated once per plan)."""
        if self._tc_scratch is None:
            from . import _native
            torch = _native.require_cuda()
            lib = _native.load()
            prep = self.prep
            a2p = (prep.A * (prep.A + 1) // 2 + 15) // 16 * 16
            per = 4 * prep.P * (prep.N + a2p)
            chunk = max(1, self.TC_CHUNK_BYTES // per)
            nbytes = int(lib.pbr_sample_eval_tc_scratch(self.struct, chunk))
            assert nbytes > 0
            self._tc_scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.tensors["vib_qq"].device)
        return self._tc_scratch
