"""The flow's CPU oracle: inverse(forward(y)) == y, log-determinants, and the analytic gradients
against central finite differences."""
import numpy as np

from oracle import flow_oracle as fo


def _setup(seed=0, D=12, L=4, H=16, X=40, A=3):
    rng = np.random.default_rng(seed)
    params = fo.init_params(D, L, H, seed=seed, scale_last=0.5)
    y = rng.normal(size=(X, D))
    mu = np.zeros((A, D))
    mu[:, 0:D:3] = rng.normal(size=(A, D // 3))
    log_w = np.log(rng.dirichlet(np.ones(A)))
    nu = rng.normal(0, 0.3, A)
    r = np.exp(rng.normal(size=X))
    return params, nu, y, r, mu, log_w


def test_inverse_undoes_forward_and_logdets_cancel():
    params, nu, y, r, mu, log_w = _setup()
    yf, ldf = fo.forward(params, y)
    yb, ldb = fo.inverse(params, yf)
    assert np.allclose(yb, y, atol=1e-10)
    assert np.allclose(ldf + ldb, 0.0, atol=1e-10)


def test_logdet_matches_numerical_jacobian():
    params, nu, y, r, mu, log_w = _setup(X=3)
    eps = 1e-6
    for i in range(3):
        J = np.zeros((y.shape[1], y.shape[1]))
        for k in range(y.shape[1]):
            yp, ym = y[i:i + 1].copy(), y[i:i + 1].copy()
            yp[0, k] += eps
            ym[0, k] -= eps
            J[:, k] = (fo.forward(params, yp)[0][0] - fo.forward(params, ym)[0][0]) / (2 * eps)
        assert np.isclose(np.log(abs(np.linalg.det(J))), fo.forward(params, y[i:i + 1])[1][0], atol=1e-6)


def test_gradients_match_finite_differences():
    params, nu, y, r, mu, log_w = _setup()
    loss, grads, g_nu = fo.loss_and_grads(params, nu, y, r, mu, log_w)
    assert np.isclose(loss, fo.loss_only(params, nu, y, r, mu, log_w))
    eps = 1e-6
    rng = np.random.default_rng(5)
    for l in (0, len(params) - 1):
        for key in ("W1", "b1", "W2", "b2", "W3", "b3"):
            arr = params[l][key]
            for _ in range(3):
                idx = tuple(rng.integers(0, n) for n in arr.shape)
                old = arr[idx]
                arr[idx] = old + eps
                lp = fo.loss_only(params, nu, y, r, mu, log_w)
                arr[idx] = old - eps
                lm = fo.loss_only(params, nu, y, r, mu, log_w)
                arr[idx] = old
                assert np.isclose(grads[l][key][idx], (lp - lm) / (2 * eps), rtol=1e-5, atol=1e-9), (l, key)
    for a in range(len(nu)):
        nu[a] += eps
        lp = fo.loss_only(params, nu, y, r, mu, log_w)
        nu[a] -= 2 * eps
        lm = fo.loss_only(params, nu, y, r, mu, log_w)
        nu[a] += eps
        assert np.isclose(g_nu[a], (lp - lm) / (2 * eps), rtol=1e-5, atol=1e-9)
