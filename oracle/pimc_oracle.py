"""FP64 numpy restatement of Pibronic's PIMC block evaluation.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the CUDA path and the timed CPU
baseline ("port") in ``bench.py --impl reference``.  Nothing in ``pibronic_gb300`` imports it;
only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may.

Every function restates one piece of the reference engine ``pibronic/pimc/pimc.py`` (the module the
reference's README calls ``pimc/minimal.py``) and cites the file:line it follows.  The arithmetic is
the reference's: FP64, numpy ``einsum`` for the coupling matrix, LAPACK ``eigh`` (lower triangle),
and a Python loop over samples x beads with two dense ``dot`` calls per bead for the ring product,
so its run time is representative of the reference's CPU path.

Random numbers follow the reference's call order on numpy's legacy global generator
(``np.random.choice`` once for all X sample sources, then one ``np.random.normal`` per block), so a
run seeded with ``np.random.seed(s)`` reproduces the reference's q stream exactly.

Parity is pinned by ``tests/test_oracle_golden.py`` against the reference's own known-answer data
(``tests/pimc/test_pimc_explicit_example.py`` + ``explicit_data/``) and against fixtures produced by
running the reference itself (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import hashlib
import json

import numpy as np

F64 = np.float64

# ---------------------------------------------------------------------------------------------
# constants (pibronic/constants.py:15-44)
# ---------------------------------------------------------------------------------------------
J_PER_EV = F64(1.6021766208e-19)              # constants.py:15
KB_EV = F64(1.38064852e-23) / J_PER_EV        # constants.py:24 (eV / K)
DELTA_BETA_DEFAULT = 2.0e-4                   # constants.py:28
HBAR = 1.0                                    # constants.py:26


def beta_of(temperature):
    """beta = 1 / (kB T) in 1/eV (constants.py:41-44)."""
    return 1.0 / (temperature * KB_EV)


# ---------------------------------------------------------------------------------------------
# model files (pibronic/vibronic/vibronic_model_io.py:42-73, 536-626)
# ---------------------------------------------------------------------------------------------
KEY_N, KEY_A = "number of modes", "number of surfaces"
KEY_E, KEY_W = "energies", "frequencies"
KEY_G1, KEY_G2 = "linear couplings", "quadratic couplings"


def model_from_text(text, diagonal=False):
    """Parse a model JSON text into FP64 arrays; a missing coupling key means all zeros
    (vibronic_model_io.py:556-572, 575-596).  Shapes: coupled E (A,A), w (N,), G1 (N,A,A),
    G2 (N,N,A,A); diagonal E (A,), G1 (N,A), G2 (N,N,A) (vibronic_model_io.py:42-73)."""
    raw = json.loads(text)
    A, N = int(raw[KEY_A]), int(raw[KEY_N])
    if diagonal:
        shapes = {KEY_E: (A,), KEY_W: (N,), KEY_G1: (N, A), KEY_G2: (N, N, A)}
    else:
        shapes = {KEY_E: (A, A), KEY_W: (N,), KEY_G1: (N, A, A), KEY_G2: (N, N, A, A)}
    out = {"A": A, "N": N}
    for key, shape in shapes.items():
        arr = np.zeros(shape, dtype=F64)
        if key in raw:
            arr[...] = np.array(raw[key], dtype=F64)
        out[key] = arr
    return out


def model_from_file(path, diagonal=False):
    with open(path, mode="r", encoding="UTF8") as fh:
        return model_from_text(fh.read(), diagonal=diagonal)


def file_hash(path):
    """SHA-512 hex digest of a model file's text (vibronic_model_io.py:293-331)."""
    with open(path, mode="r", encoding="UTF8") as fh:
        return hashlib.sha512(fh.read().encode("UTF-8")).hexdigest()


# ---------------------------------------------------------------------------------------------
# temperature dependent constants (pimc.py:59-89)
# ---------------------------------------------------------------------------------------------
def temperature_constants(omega, n_states, tilde_energy, tau):
    """coth(tau w), csch(tau w) broadcast to (A,N) and the per-surface O-matrix prefactor
    exp(-tau Etilde_a) * prod_j csch_aj^(1/2) (pimc.py:61-81)."""
    w = np.broadcast_to(omega, (n_states, omega.shape[0]))
    coth = np.tanh(HBAR * tau * w) ** (-1.0)
    csch = np.sinh(HBAR * tau * w) ** (-1.0)
    prefactor = np.exp(-tau * tilde_energy) * np.prod(csch, axis=1) ** 0.5
    return {"coth": coth, "csch": csch, "prefactor": prefactor, "tau": tau}


# ---------------------------------------------------------------------------------------------
# model preparation (pimc.py:172-235 vibronic, 251-269 plus/minus, 282-424 sampling)
# ---------------------------------------------------------------------------------------------
def prepare_vibronic(model, beta, beads, delta_beta=None):
    """Fold the diagonal linear terms and diagonal energies of the coupled model into the
    harmonic oscillators (pimc.py:172-177, 208-235): Delta_a = -1/2 sum_j L_jaa^2 / w_j,
    d_a = -L_jaa / w_j, then zero diag(L) and diag(E).  With delta_beta, also the beta +- dbeta
    constants (pimc.py:251-269)."""
    A, N = model["A"], model["N"]
    w = model[KEY_W].copy()
    E = model[KEY_E].copy()
    L = model[KEY_G1].copy()
    Q = model[KEY_G2].copy()
    lin_diag = np.array([L[:, a, a] for a in range(A)])          # (A, N)
    delta = -0.5 * (lin_diag ** 2.0 / w[None, :]).sum(axis=1)   # pimc.py:176
    tilde = np.diag(E) + delta                                   # pimc.py:75-76
    tau = beta / beads
    out = {"A": A, "N": N, "omega": w, "delta": delta, "tilde_energy": tilde,
           "const": temperature_constants(w, A, tilde, tau)}
    if delta_beta is not None:
        out["const_plus"] = temperature_constants(w, A, tilde, (beta + delta_beta) / beads)
        out["const_minus"] = temperature_constants(w, A, tilde, (beta - delta_beta) / beads)
    shift = -lin_diag / w[None, :]                               # pimc.py:212
    for a in range(A):                                           # pimc.py:214-217
        L[:, a, a] = 0.0
        E[a, a] = 0.0
    out.update(state_shift=shift, energy=E, linear=L, quadratic=Q)
    return out


def prepare_sampling(model, beta, beads, samples, circ_eigvals, draw_sources=True):
    """Diagonal sampling model rho (pimc.py:282-424): Delta_a from the linear terms, normalised
    state weights w_a ~ exp(-beta (E_a + Delta_a)) / prod_j sinh(beta w_j / 2) (pimc.py:343-350),
    d_a = -L_ja / w_j, the X sample sources drawn up front with np.random.choice
    (pimc.py:386-389), and the normal-mode precision 2 coth_aj - csch_aj lambda_k
    (pimc.py:402-404).  Quadratic terms of rho are ignored, as in the reference."""
    A, N = model["A"], model["N"]
    w = model[KEY_W].copy()
    lin = model[KEY_G1].copy()                                   # (N, A)
    delta = -0.5 * (lin ** 2.0 / w[:, None]).sum(axis=0)         # pimc.py:338
    weight = np.exp(-beta * (model[KEY_E] + delta))              # pimc.py:343
    weight /= np.prod(np.sinh((beta * w) / 2.0))                 # pimc.py:347
    weight /= weight.sum()                                       # pimc.py:350
    tau = beta / beads
    tilde = model[KEY_E] + delta
    const = temperature_constants(w, A, tilde, tau)
    shift = (-lin / w[:, None]).T.copy()                         # (A, N) pimc.py:376
    out = {"A": A, "N": N, "omega": w, "delta": delta, "state_weight": weight,
           "tilde_energy": tilde, "const": const, "state_shift": shift}
    if draw_sources:
        out["sample_sources"] = np.random.choice(range(A), size=samples, p=weight)  # pimc.py:386
    invcov = 2.0 * const["coth"][:, :, None] - const["csch"][:, :, None] * circ_eigvals[None, None, :]
    out["inverse_covariance"] = invcov                           # (A, N, P) pimc.py:402
    return out


def circulant_basis(beads):
    """Ring adjacency circulant C with first column [0,1,0,...,0,1] and its eigen-decomposition
    (pimc.py:683-689); requires P >= 3."""
    assert beads >= 3, "circulant matrix requires 3 or more beads"
    first = np.zeros(beads)
    first[1] = first[-1] = 1.0
    idx = (np.arange(beads)[:, None] - np.arange(beads)[None, :]) % beads
    C = first[idx]
    vals, vecs = np.linalg.eigh(C, UPLO="L")
    return C, vals, vecs


# ---------------------------------------------------------------------------------------------
# sampling (pimc.py:326-334, 613-631, 602-611)
# ---------------------------------------------------------------------------------------------
def draw_normal_modes(rho, sample_view, beads):
    """cc ~ Normal(0, 1/sqrt(invcov[source])) with shape (B,N,P) (pimc.py:326-334, 404)."""
    src = rho["sample_sources"][sample_view]
    std = np.sqrt(1.0 / rho["inverse_covariance"][src, ...])
    return np.random.normal(loc=np.zeros(std.shape), scale=std, size=std.shape)


def transform_to_beads(cc, circ_vecs, rho, sample_view):
    """q[b,j,p] = sum_k V[p,k] cc[b,j,k] + d_src(b),j  (pimc.py:618-624); shape (B,N,P)."""
    q = np.einsum("ab,ijb->ija", circ_vecs, cc)
    src = rho["sample_sources"][sample_view]
    q += rho["state_shift"][src, :, None]
    return q


# ---------------------------------------------------------------------------------------------
# stage functions (pimc.py:1062-1213)
# ---------------------------------------------------------------------------------------------
def o_matrix(q_slots, state_shift, const, n_fill):
    """Dense (B,P,A,A) O matrices with only the diagonal set (pimc.py:1087-1129):
    O[b,p,a,a] = prefactor_a * exp(-1/2 sum_j [coth_aj (x_p^2 + x_{p+1}^2) - 2 csch_aj x_p x_{p+1}])
    with x = q - d_a and the ring closed by np.roll.  ``q_slots`` is (B, A_m, N, P) (one slot per
    surface of this model); only the first ``n_fill`` diagonal entries are written
    (pimc.py:1110-1111 fills data.states entries even when the model has more)."""
    B, A_m, N, P = q_slots.shape
    x1 = q_slots - state_shift[None, :, :, None]
    x2 = np.roll(x1, shift=-1, axis=3)
    coth = const["coth"][None, :, :, None]
    csch = const["csch"][None, :, :, None]
    expo = -0.5 * np.sum(coth * (x1 ** 2.0 + x2 ** 2.0) - 2.0 * csch * x1 * x2, axis=2)  # (B,A,P)
    expo = np.exp(expo).swapaxes(1, 2)                                                  # (B,P,A)
    out = np.zeros((B, P, A_m, A_m), dtype=F64)
    for a in range(n_fill):
        out[:, :, a, a] = expo[:, :, a]
    out *= const["prefactor"][None, None, :, None]
    return out


def scaling_factors(o_one, o_two):
    """S12[b,p] = max(max O1[b,p], max O2[b,p]) (pimc.py:1076-1084)."""
    return np.maximum(np.amax(o_one, axis=(2, 3)), np.amax(o_two, axis=(2, 3)))


def denominator(o_rho):
    """rho[b] = Tr prod_p O^rho[b,p] (pimc.py:1132-1136)."""
    return o_rho.prod(axis=1).trace(axis1=1, axis2=2)


def coupling_matrix(q_slots, vib):
    """V[b,p,x,y] = sum_{d,e} q[b,y,e,p] 1/2 Q[d,e,x,y] q[b,x,d,p] + sum_d L[d,x,y] q[b,x,d,p] + E[x,y]
    (pimc.py:1147-1160, einsums 'acef,debc,abdf->afbc' and 'dbc,abdf->afbc'); symmetric check
    as pimc.py:1169."""
    V = np.einsum("acef,debc,abdf->afbc", q_slots, 0.5 * vib["quadratic"], q_slots)
    V += np.einsum("dbc,abdf->afbc", vib["linear"], q_slots)
    V += vib["energy"][None, None, :, :]
    assert np.allclose(V.transpose(0, 1, 3, 2), V)
    return V


def m_matrix(V, tau):
    """M = U diag(exp(-tau lambda)) U^T from LAPACK eigh on the lower triangle, with the
    central tau (pimc.py:1171-1187)."""
    lam, U = np.linalg.eigh(V, UPLO="L")
    return np.einsum("abcd,abd,abed->abce", U, np.exp(-tau * lam), U, optimize="optimal")


def numerator(M, O):
    """g[b] = Tr prod_p (M_p O_p), a Python loop over samples and beads with two dense dots per
    bead, exactly the reference's evaluation order (pimc.py:1194-1209)."""
    B, P, A, _ = M.shape
    g = np.empty(B, dtype=F64)
    eye = np.identity(A)
    for b in range(B):
        acc = eye.copy()
        for p in range(P):
            acc = acc.dot(M[b, p])
            acc = acc.dot(O[b, p])
        g[b] = np.trace(acc)
    return g


# ---------------------------------------------------------------------------------------------
# the box: preprocess + block drivers (pimc.py:647-738, 1341-1462, 1216-1338)
# ---------------------------------------------------------------------------------------------
class OracleBox:
    """Holds what ``BoxData(PM).preprocess`` builds (pimc.py:647-738)."""

    def __init__(self, vib_model, rho_model, samples, block_size, beads, temperature,
                 delta_beta=None, draw_sources=True):
        self.samples, self.block_size, self.beads = samples, block_size, beads
        self.blocks = samples // block_size
        self.temperature = temperature
        self.beta = beta_of(temperature)
        self.tau = self.beta / beads
        self.delta_beta = delta_beta
        self.A, self.N = vib_model["A"], vib_model["N"]
        self.C, self.circ_vals, self.circ_vecs = circulant_basis(beads)
        self.vib = prepare_vibronic(vib_model, self.beta, beads, delta_beta)
        self.rho = prepare_sampling(rho_model, self.beta, beads, samples, self.circ_vals,
                                    draw_sources=draw_sources)
        self.A_rho = self.rho["A"]

    # -- per-block helpers ------------------------------------------------------------------
    def draw_q(self, sample_view):
        """One block of bead coordinates (B,N,P), the reference's draw + transform."""
        cc = draw_normal_modes(self.rho, sample_view, self.beads)
        return transform_to_beads(cc, self.circ_vecs, self.rho, sample_view)

    def slots(self, q, n):
        return np.broadcast_to(q[:, None, :, :], (q.shape[0], n) + q.shape[1:]).copy()

    def evaluate(self, q, plus_minus=True, scaled=True):
        """Everything the block loop does after sampling (pimc.py:1430-1449) for given q (B,N,P).
        Returns dict with rho, g (and gP, gM), all scaled by prod_p 1/S12 when ``scaled``."""
        qv = self.slots(q, self.A)
        qr = qv if self.A_rho == self.A else self.slots(q, self.A_rho)
        o_rho = o_matrix(qr, self.rho["state_shift"], self.rho["const"], min(self.A, self.A_rho))
        o_vib = o_matrix(qv, self.vib["state_shift"], self.vib["const"], self.A)
        S12 = scaling_factors(o_rho, o_vib) if scaled else np.ones(q.shape[:1] + (self.beads,))
        o_rho /= S12[..., None, None]
        o_vib /= S12[..., None, None]
        out = {"S12": S12, "o_rho": o_rho, "o_vib": o_vib}
        out["rho"] = denominator(o_rho)
        V = coupling_matrix(qv, self.vib)
        M = m_matrix(V, self.tau)
        out["M"] = M
        out["g"] = numerator(M, o_vib)
        if plus_minus:
            for key, ck in (("gP", "const_plus"), ("gM", "const_minus")):
                o_pm = o_matrix(qv, self.vib["state_shift"], self.vib[ck], self.A)
                o_pm /= S12[..., None, None]
                out[key] = numerator(M, o_pm)
        return out

    def block_compute(self, plus_minus=True):
        """block_compute_pm / block_compute (pimc.py:1388-1462, 1341-1385) -> per-sample scaled
        outputs as the .npz keys s_rho, s_g (, s_gP, s_gM) and the q of every sample."""
        X = self.blocks * self.block_size
        res = {k: np.full(self.samples, np.nan) for k in
               (("s_rho", "s_g", "s_gP", "s_gM") if plus_minus else ("s_rho", "s_g"))}
        qs = np.empty((X, self.N, self.beads))
        for blk in range(self.blocks):
            view = slice(blk * self.block_size, (blk + 1) * self.block_size)
            q = self.draw_q(view)
            qs[view] = q
            ev = self.evaluate(q, plus_minus=plus_minus)
            res["s_rho"][view] = ev["rho"]
            res["s_g"][view] = ev["g"]
            if plus_minus:
                res["s_gP"][view] = ev["gP"]
                res["s_gM"][view] = ev["gM"]
        res["q"] = qs
        return res

    # -- learned-proposal data path (pimc.py:602-611, 1273-1338) ------------------------------
    def g_of_R(self, R):
        """g(R) for given dimensionless R (B,N,P): the slots hold q = R - d_a and the O matrix
        shifts again by d_a (pimc.py:606-610, 1327-1334); unscaled."""
        slots = R[:, None, :, :] - self.vib["state_shift"][None, :, :, None]
        o_vib = o_matrix(slots, self.vib["state_shift"], self.vib["const"], self.A)
        V = coupling_matrix(slots, self.vib)
        return numerator(m_matrix(V, self.tau), o_vib)

    def rho_of_R(self, R):
        """rho(R) for given R (B,N,P) (pimc.py:1273-1302); unscaled.  The slots are R - d^vib_a
        and the rho O matrix reads them, which the reference only does when A_rho == A (with
        A_rho != A it reads a scratch tensor this path never fills, pimc.py:1091-1096)."""
        assert self.A_rho == self.A, "rho(R) needs a sampling model with the vibronic surface count"
        slots = R[:, None, :, :] - self.vib["state_shift"][None, :, :, None]
        o_rho = o_matrix(slots, self.rho["state_shift"], self.rho["const"],
                         min(self.A, self.A_rho))
        return denominator(o_rho)
