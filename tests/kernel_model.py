"""Numpy model of the fused kernel's arithmetic (test infrastructure).

Evaluates, in FP64 on the CPU, exactly the formulation the CUDA kernel uses with the tables that
pibronic_gb300.plan builds: the cancellation-free O-matrix exponent, ln S12 in log space, the
Taylor series in the beta step for g(beta +- db), M = exp(-tau V) by eigh.  Comparing it with
the oracle checks the formulation independently of the GPU.
"""
import numpy as np

from pibronic_gb300.plan import pair_index


def evaluate(prep, q):
    """q: (X, N, P) FP64 -> dict s_rho, s_g, s_gp, s_gm, coef (X, K+1)."""
    t = prep.tables()
    A, N, P, K = prep.A, prep.N, prep.P, prep.K
    X = q.shape[0]
    cs = t["vib_cs"].reshape(K + 1, N)
    th = t["vib_th"].reshape(K + 1, N)
    cc = t["vib_c"].reshape(K + 1, A)
    d = t["vib_d"].reshape(A, N)
    rd = t["rho_d"].reshape(-1, N)[:A]
    qn = np.roll(q, -1, axis=2)
    dq2 = (q - qn) ** 2                                              # (X,N,P)
    # vib exponent series (X,P,K+1,A)
    ua = q[:, None, :, :] - d[None, :, :, None]                      # (X,A,N,P)
    ub = qn[:, None, :, :] - d[None, :, :, None]
    S = ua ** 2 + ub ** 2
    phv = (cc[None, None, :, :]
           - np.einsum("kj,xjp->xpk", cs, dq2)[:, :, :, None]
           - np.einsum("kj,xajp->xpka", th, S))
    ra = q[:, None, :, :] - rd[None, :, :, None]
    rb = qn[:, None, :, :] - rd[None, :, :, None]
    phr = (t["rho_c"][:A][None, None, :]
           - np.einsum("j,xjp->xp", t["rho_cs"], dq2)[:, :, None]
           - np.einsum("j,xajp->xpa", t["rho_th"], ra ** 2 + rb ** 2))
    lmax = np.maximum(phv[:, :, 0, :].max(axis=2), phr.max(axis=2))  # (X,P)
    s_rho = np.exp((phr - lmax[:, :, None]).sum(axis=1)).sum(axis=1)
    # O series: exp(phi0 - lmax) * exp(sum_{k>=1} phi_k h^k)
    E = np.zeros((X, P, K + 1, A))
    E[:, :, 0, :] = 1.0
    for k in range(1, K + 1):
        acc = np.zeros((X, P, A))
        for i in range(1, k + 1):
            acc += i * phv[:, :, i, :] * E[:, :, k - i, :]
        E[:, :, k, :] = acc / k
    O = np.exp(phv[:, :, 0, :] - lmax[:, :, None])[:, :, None, :] * E   # (X,P,K+1,A)
    # V from the packed tables
    A2 = A * (A + 1) // 2
    e = t["vib_e"]
    lt = t["vib_l"].reshape(N, A2)
    qq = t["vib_qq"].reshape(N * (N + 1) // 2, A2)
    prs = np.array([q[:, dd, :] * q[:, ee, :] for dd in range(N) for ee in range(dd + 1)])  # (N2,X,P)
    vp = e[None, None, :] + np.einsum("jr,xjp->xpr", lt, q) + np.einsum("nr,nxp->xpr", qq, prs)
    V = np.zeros((X, P, A, A))
    for b in range(A):
        for c in range(b + 1):
            V[:, :, b, c] = V[:, :, c, b] = vp[:, :, pair_index(b, c)]
    lam, U = np.linalg.eigh(V)
    M = np.einsum("xpij,xpj,xpkj->xpik", U, np.exp(-prep.tau * lam), U)
    # ring product with the series
    Nser = np.zeros((X, K + 1, A, A))
    Nser[:, 0] = np.eye(A)
    for p in range(P):
        Y = np.einsum("xkij,xjl->xkil", Nser, M[:, p])
        new = np.zeros_like(Nser)
        for k in range(K + 1):
            for i in range(k + 1):
                new[:, k] += Y[:, i] * O[:, p, k - i, None, :]
        Nser = new
    coef = np.trace(Nser, axis1=2, axis2=3)                          # (X,K+1)
    db = prep.delta_beta
    powers = db ** np.arange(K + 1)
    out = {"s_rho": s_rho, "s_g": coef[:, 0], "coef": coef}
    if K > 0:
        out["s_gp"] = coef @ powers
        out["s_gm"] = coef @ (powers * (-1.0) ** np.arange(K + 1))
    return out
