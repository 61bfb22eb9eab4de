"""Seeded synthetic vibronic models in the reference's JSON format.

Recipe (the shapes and value distributions of the benchmark configurations):
  frequencies w_j ~ U[0.02, 0.30] eV; diagonal energies ~ U[0, 0.5] eV; symmetric off-diagonal
  energies ~ N(0, sd_offdiag); linear couplings ~ N(0, 0.01) symmetrised in the surfaces;
  quadratic couplings ~ N(0, sd_quadratic) symmetrised in the modes and in the surfaces, then
  shrunk until 1/2 diag(w) + Q_aa is positive definite (margin: smallest eigenvalue at least
  w_min / 8) for every surface.  The sampling model rho is the diagonal (harmonic) part of the
  coupled model (vibronic_model_io.py:774-787).
"""
from __future__ import annotations

import os

import numpy as np

from . import vibronic_io as vIO
from .vibronic_io import VMK


def make_coupled_model(A, N, seed, sd_offdiag=0.05, sd_linear=0.01, sd_quadratic=0.002,
                       quadratic=True):
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.02, 0.30, size=N)
    E = np.zeros((A, A))
    E[np.diag_indices(A)] = rng.uniform(0.0, 0.5, size=A)
    off = rng.normal(0.0, sd_offdiag, size=(A, A))
    iu = np.triu_indices(A, 1)
    E[iu] = off[iu]
    E[(iu[1], iu[0])] = off[iu]
    L = rng.normal(0.0, sd_linear, size=(N, A, A))
    L = 0.5 * (L + L.transpose(0, 2, 1))
    Q = np.zeros((N, N, A, A))
    if quadratic and sd_quadratic > 0:
        Q = rng.normal(0.0, sd_quadratic, size=(N, N, A, A))
        Q = 0.5 * (Q + Q.transpose(1, 0, 2, 3))
        Q = 0.5 * (Q + Q.transpose(0, 1, 3, 2))
        margin = w.min() / 8.0
        for _ in range(200):
            ok = all(np.linalg.eigvalsh(0.5 * np.diag(w) + Q[:, :, a, a]).min() >= margin
                     for a in range(A))
            if ok:
                break
            Q *= 0.8
    return {VMK.N: N, VMK.A: A, VMK.E: E, VMK.w: w, VMK.G1: L, VMK.G2: Q}


def make_near_degenerate_model(A, N, seed, eps=1e-7, sd_quadratic=0.002):
    """A coupled model whose surfaces are degenerate up to couplings of size eps (eV): every
    surface has the same energy, linear and quadratic diagonal terms (those of surface 0 of the
    recipe above), and the off-diagonal energies, linear and quadratic couplings are N(0, eps).
    V(q) is then v0(q) I + O(eps) at every q: its eigenvalues coincide to ~eps and its eigenvectors
    are ill-conditioned, while exp(-tau V) is not (the reference forms it with LAPACK eigh,
    pimc.py:1171-1173)."""
    base = make_coupled_model(A, N, seed, sd_quadratic=sd_quadratic)
    rng = np.random.default_rng(seed + 7)
    eye = np.eye(A)

    def sym_noise(shape):
        x = rng.normal(0.0, eps, size=shape)
        x = 0.5 * (x + np.swapaxes(x, -1, -2))
        return x * (1.0 - eye)

    E = base[VMK.E][0, 0] * eye + sym_noise((A, A))
    L = base[VMK.G1][:, 0, 0][:, None, None] * eye + sym_noise((N, A, A))
    Qn = sym_noise((N, N, A, A))
    Qn = 0.5 * (Qn + Qn.transpose(1, 0, 2, 3))
    Q = base[VMK.G2][:, :, 0, 0][:, :, None, None] * eye + Qn
    return {VMK.N: N, VMK.A: A, VMK.E: E, VMK.w: base[VMK.w], VMK.G1: L, VMK.G2: Q}


def diagonal_of(model):
    out = {VMK.N: model[VMK.N], VMK.A: model[VMK.A]}
    for key in (VMK.E, VMK.w, VMK.G1, VMK.G2):
        v = model[key]
        out[key] = np.diagonal(v, axis1=v.ndim - 2, axis2=v.ndim - 1).copy() if v.ndim >= 2 else v.copy()
    return out


def write_model_pair(FS, A, N, seed, **kw):
    """Write coupled_model.json and the basic sampling_model.json of FS; returns the coupled dict."""
    model = make_coupled_model(A, N, seed, **kw)
    os.makedirs(os.path.dirname(FS.path_vib_model), exist_ok=True)
    vIO.save_model_to_JSON(FS.path_vib_model, model)
    vIO.create_basic_diagonal_model(FS)
    return model


def batch_models(count=256, seed=3, A_range=(2, 8), N_range=(3, 20), P_range=(8, 256), T_range=(100.0, 500.0),
                 rel_delta_beta=1e-4):
    """Seeded independent models of uneven sizes for the batched configuration: A ~ U{2..8},
    N ~ U{3..20}, P ~ U{8..256}, T ~ U[100, 500] K, each with the coupled-model recipe above and
    rho its diagonal.  Returns PreparedModels (beta +- rel_delta_beta * beta series)."""
    from .constants import beta as beta_of
    from .plan import PreparedModels
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        A = int(rng.integers(A_range[0], A_range[1] + 1))
        N = int(rng.integers(N_range[0], N_range[1] + 1))
        P = int(rng.integers(P_range[0], P_range[1] + 1))
        T = float(rng.uniform(*T_range))
        m = make_coupled_model(A, N, seed * 100003 + i)
        b = beta_of(T)
        out.append(PreparedModels(m, diagonal_of(m), P, beta=b, delta_beta=rel_delta_beta * b))
    return out


#: benchmark configurations (sizes of the reference's headline runs)
CONFIGS = {
    1: dict(A=2, N=2, P=12, T=300.0, X=10_000, B=1_000),
    2: dict(A=4, N=12, P=64, T=300.0, X=1_000_000, B=10_000),
}
