"""FP64 numpy reference of the learned proposal (affine-coupling flow).  TEST INFRASTRUCTURE ONLY:
the checker for pibronic_gb300.flow's CUDA kernels (forward, inverse, loss, gradients).

The proposal acts on D = N * nsel whitened ring normal-mode coordinates y (for every mode j the
slots s = 0 .. nsel-1 of the real Fourier ring basis, divided by their rho standard deviation);
every other coordinate keeps rho's distribution.  Base density on y: the mixture
sum_a pi_a N(y; mu_a, I), pi = softmax(log w + nu) (w the rho state weights, nu learned), mu_a the
whitened state shifts (non-zero only in the centroid slot).  Coupling layer l (mask: even layers
transform the odd positions, odd layers the even ones):
    forward  y_B' = y_B * exp(s) + t,   inverse y_B = (y_B' - t) * exp(-s),
    (s, t) = head(tanh(tanh(y_A W1 + b1) W2 + b2) W3 + b3),  s = kappa * tanh(raw_s / kappa).
Training minimises the forward KL to the target weighted by r = g/rho of rho's own samples:
    L = - sum_i rt_i [log M(f^-1(y_i)) + log|det d f^-1 / dy|(y_i)],  rt = r / sum r.
"""
from __future__ import annotations

import numpy as np

KAPPA = 2.0


def masks(D, layers):
    """(A indices, B indices) per layer: even layers condition on even positions."""
    idx = np.arange(D)
    out = []
    for l in range(layers):
        a, b = (idx[0::2], idx[1::2]) if l % 2 == 0 else (idx[1::2], idx[0::2])
        out.append((a, b))
    return out


def init_params(D, layers, hidden, seed=0, scale_last=0.0):
    rng = np.random.default_rng(seed)
    ps = []
    for (a, b) in masks(D, layers):
        I, J = len(a), len(b)
        ps.append({
            "W1": rng.normal(0, 1 / np.sqrt(I), (I, hidden)), "b1": np.zeros(hidden),
            "W2": rng.normal(0, 1 / np.sqrt(hidden), (hidden, hidden)), "b2": np.zeros(hidden),
            "W3": rng.normal(0, scale_last / np.sqrt(hidden), (hidden, 2 * J)), "b3": np.zeros(2 * J),
        })
    return ps


def _net(p, ya):
    h1 = np.tanh(ya @ p["W1"] + p["b1"])
    h2 = np.tanh(h1 @ p["W2"] + p["b2"])
    o = h2 @ p["W3"] + p["b3"]
    J = o.shape[1] // 2
    s = KAPPA * np.tanh(o[:, :J] / KAPPA)
    return h1, h2, s, o[:, J:]


def forward(params, y):
    """Sampling direction: y -> y', log|det dy'/dy|."""
    D = y.shape[1]
    y = y.copy()
    logdet = np.zeros(y.shape[0])
    for p, (a, b) in zip(params, masks(D, len(params))):
        _, _, s, t = _net(p, y[:, a])
        y[:, b] = y[:, b] * np.exp(s) + t
        logdet += s.sum(axis=1)
    return y, logdet


def inverse(params, y, keep=False):
    """Training direction: y' -> y, log|det dy/dy'|; with keep, the per-layer intermediates."""
    D = y.shape[1]
    y = y.copy()
    logdet = np.zeros(y.shape[0])
    tape = []
    mk = masks(D, len(params))
    for l in range(len(params) - 1, -1, -1):
        p, (a, b) = params[l], mk[l]
        ya = y[:, a].copy()
        h1, h2, s, t = _net(p, ya)
        yb = (y[:, b] - t) * np.exp(-s)
        tape.append((l, ya, h1, h2, s, t, yb))
        y[:, b] = yb
        logdet -= s.sum(axis=1)
    return (y, logdet, tape) if keep else (y, logdet)


def base_logpdf(y, mu, log_pi):
    """log sum_a pi_a exp(-|y - mu_a|^2 / 2) (no 2 pi constant) and responsibilities."""
    e = log_pi[None, :] - 0.5 * ((y[:, None, :] - mu[None, :, :]) ** 2).sum(axis=2)
    m = e.max(axis=1, keepdims=True)
    lse = m[:, 0] + np.log(np.exp(e - m).sum(axis=1))
    return lse, np.exp(e - lse[:, None])


def log_pi_of(log_w, nu):
    z = log_w + nu
    return z - (z.max() + np.log(np.exp(z - z.max()).sum()))


def loss_and_grads(params, nu, y, r, mu, log_w):
    """Weighted forward-KL loss and its gradients (analytic back-propagation)."""
    rt = r / r.sum()
    log_pi = log_pi_of(log_w, nu)
    y0, ld, tape = inverse(params, y, keep=True)
    lse, gam = base_logpdf(y0, mu, log_pi)
    loss = -np.sum(rt * (lse + ld))
    pi = np.exp(log_pi)
    g_nu = -np.sum(rt[:, None] * (gam - pi[None, :]), axis=0)
    gy = rt[:, None] * np.einsum("ia,iad->id", gam, y0[:, None, :] - mu[None, :, :])
    D = y.shape[1]
    mk = masks(D, len(params))
    grads = [None] * len(params)
    for (l, ya, h1, h2, s, t, yb) in reversed(tape):      # layers 0 .. L-1
        p, (a, b) = params[l], mk[l]
        gyb = gy[:, b]
        es = np.exp(-s)
        g_in_b = gyb * es
        g_t = -gyb * es
        g_s = -gyb * yb + rt[:, None]
        g_os = g_s * (1 - (s / KAPPA) ** 2)
        g_o = np.concatenate([g_os, g_t], axis=1)
        gW3 = h2.T @ g_o
        gb3 = g_o.sum(axis=0)
        g_z2 = (g_o @ p["W3"].T) * (1 - h2 ** 2)
        gW2 = h1.T @ g_z2
        gb2 = g_z2.sum(axis=0)
        g_z1 = (g_z2 @ p["W2"].T) * (1 - h1 ** 2)
        gW1 = ya.T @ g_z1
        gb1 = g_z1.sum(axis=0)
        g_ya = g_z1 @ p["W1"].T
        new = gy.copy()
        new[:, a] = gy[:, a] + g_ya
        new[:, b] = g_in_b
        gy = new
        grads[l] = {"W1": gW1, "b1": gb1, "W2": gW2, "b2": gb2, "W3": gW3, "b3": gb3}
    return loss, grads, g_nu


def loss_only(params, nu, y, r, mu, log_w):
    rt = r / r.sum()
    y0, ld = inverse(params, y)
    lse, _ = base_logpdf(y0, mu, log_pi_of(log_w, nu))
    return -np.sum(rt * (lse + ld))
