"""Learned importance proposal: an affine-coupling flow over whitened ring normal modes, trained and
applied with the library's own CUDA kernels (pbr_flow_*, pbr_gemm_tn_acc, pbr_adam).

Coordinates.  For every mode j the first ``nsel`` slots of the real Fourier ring basis (centroid,
then the cos/sin pairs of the lowest frequencies) are whitened by rho's standard deviation:
y_js = B_s^T (q_j - c_j) / sigma_js.  Every other direction keeps rho's distribution.

Proposal.  Base sample q ~ rho with the surface drawn from pi = softmax(log w + nu) (w: rho's
state weights, nu learned); y' = f(y) through ``layers`` coupling layers; x = q + B sigma (y' - y).
Its exact density at x is q_flow(x) = rho_nu(q) / |det df/dy|, so w = g(x) / q_flow(x) is an
unbiased importance weight for any parameters, and nu = 0 with zero last-layer weights is rho
itself (the fallback).  Training minimises the forward KL to the target on weighted samples the
method generates itself: rho's samples with weights g/rho, then the proposal's own samples with
weights g/q_flow.
"""
from __future__ import annotations

import math

import numpy as np

from . import _native
from .plan import ring_mode_eigenvalues

KAPPA = 2.0


def _lib():
    return _native.load()


class FlowProposal:
    def __init__(self, prep, plan, nsel=3, layers=8, hidden=128, seed=0, init_scale=0.0):
        torch = _native.require_cuda()
        self.prep, self.plan = prep, plan
        self.N, self.P, self.nsel = prep.N, prep.P, nsel
        self.D = prep.N * nsel
        self.layers, self.H = layers, hidden
        dev = torch.device("cuda", torch.cuda.current_device())
        self.dev = dev
        assert prep.A_rho == prep.A, "the learned proposal needs a sampling model with the coupled surface count"
        A = prep.n_fill_rho
        self.A = A
        tau, P = prep.tau, prep.P
        w_all = prep.state_weight
        # whitening constants
        lam = ring_mode_eigenvalues(P)[:nsel]
        coth = 1.0 / np.tanh(tau * prep.rho_omega)
        csch = 1.0 / np.sinh(tau * prep.rho_omega)
        sigma = 1.0 / np.sqrt(2.0 * coth[:, None] - csch[:, None] * lam[None, :])   # (N, nsel)
        center = (w_all[:, None] * prep.rho_shift).sum(axis=0)                      # (N,)
        mu = np.zeros((A, self.N, nsel))
        mu[:, :, 0] = math.sqrt(P) * (prep.rho_shift[:A] - center[None, :]) / sigma[None, :, 0]
        # rho's absolute log mixture weights in the selected coordinates: log C_a = P ln pref_a
        tabs = prep.tables()
        log_c = P * (np.asarray(tabs["rho_c"][:A], dtype=np.float64) + tabs["log_c0"])
        self.log_w = np.log(w_all[:A] / w_all[:A].sum())
        self.log_k = log_c - self.log_w                 # log C_a - log w_a (equal for all a)
        f64 = dict(dtype=torch.float64, device=dev)
        self.t_center = torch.as_tensor(center, **f64)
        self.t_sigma = torch.as_tensor(sigma.ravel(), **f64)
        self.t_inv_sigma = torch.as_tensor(1.0 / sigma.ravel(), **f64)
        self.t_csch = torch.as_tensor(csch, **f64)
        self.t_tanh2 = torch.as_tensor(np.tanh(0.5 * tau * prep.rho_omega), **f64)
        self.t_mu = torch.as_tensor(mu.reshape(A, self.D), dtype=torch.float32, device=dev)
        # parameters
        rng = np.random.default_rng(seed)
        idx = np.arange(self.D)
        self.idx = []
        init = []
        for l in range(layers):
            a, b = (idx[0::2], idx[1::2]) if l % 2 == 0 else (idx[1::2], idx[0::2])
            I, J = len(a), len(b)
            init.append({
                "W1": rng.normal(0, 1 / math.sqrt(I), (I, hidden)), "b1": np.zeros(hidden),
                "W2": rng.normal(0, 1 / math.sqrt(hidden), (hidden, hidden)), "b2": np.zeros(hidden),
                "W3": rng.normal(0, init_scale / math.sqrt(hidden), (hidden, 2 * J)), "b3": np.zeros(2 * J),
            })
            self.idx.append((torch.as_tensor(a, dtype=torch.int32, device=dev),
                             torch.as_tensor(b, dtype=torch.int32, device=dev)))
        # every parameter (and nu) is a view into one flat FP32 buffer, the gradients into a second
        # one of the same layout: the Adam update is a single launch; segments start on 16 bytes
        self._segs, n = [], 0
        for p in init:
            seg = {}
            for k, v in p.items():
                seg[k] = (n, v.shape)
                n += (v.size + 3) // 4 * 4
            self._segs.append(seg)
        self._nu_off = n
        n += (A + 3) // 4 * 4
        self._flat = torch.zeros(n, dtype=torch.float32, device=dev)
        self._gflat = torch.zeros_like(self._flat)
        self.params = [self._views(self._flat, l) for l in range(layers)]
        for p, v in zip(self.params, init):
            for k in p:
                p[k].copy_(torch.as_tensor(v[k], dtype=torch.float32))
        self.nu = self._flat[self._nu_off:self._nu_off + A]
        self._t_log_w = torch.as_tensor(self.log_w, dtype=torch.float32, device=dev)
        self._adam = None
        # the sampling direction on the tensor cores (BF16 weights, FP32 coupling and log-det)
        # where every layer's shape allows it; sample_and_evaluate uses it by default
        lib = _lib()
        self._tc_bytes = [int(lib.pbr_flow_tc_packed_bytes(self.D, int(a.numel()), int(b.numel()), hidden))
                          for a, b in self.idx]
        self.sample_tc = all(n > 0 for n in self._tc_bytes)
        self._tc_packs = None
        self._step = torch.zeros(1, dtype=torch.int32, device=dev)       # Adam's step count

    def _views(self, flat, l):
        return {k: flat[o:o + int(np.prod(shp))].view(*shp) for k, (o, shp) in self._segs[l].items()}

    # ------------------------------------------------------------------------------------------
    def layer_struct(self, l):
        p, (a, b) = self.params[l], self.idx[l]
        s = _native.PbrFlowLayer()
        s.D, s.I, s.J, s.H = self.D, int(a.numel()), int(b.numel()), self.H
        s.idx_a, s.idx_b = a.data_ptr(), b.data_ptr()
        for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
            setattr(s, k, p[k].data_ptr())
        return s

    def log_pi(self):
        torch = _native.require_cuda()
        z = self._t_log_w + self.nu
        return z - torch.logsumexp(z, dim=0)

    def params_host(self):
        return [{k: v.double().cpu().numpy() for k, v in p.items()} for p in self.params]

    # ------------------------------------------------------------------------------------------
    def prepare(self, q):
        """Selected whitened coordinates y [X, D] and the rest of rho's quadratic form U [X]."""
        torch = _native.require_cuda()
        X = q.shape[0]
        y = torch.empty((X, self.D), dtype=torch.float32, device=self.dev)
        U = torch.empty(X, dtype=torch.float64, device=self.dev)
        p = _native.ptr
        _native.check(_lib().pbr_flow_prepare(p(q), X, self.N, self.P, self.nsel, p(self.t_center),
                                              p(self.t_inv_sigma), p(self.t_csch), p(self.t_tanh2),
                                              p(y), p(U), _native.stream_handle()), "flow_prepare")
        return y, U

    def forward(self, y):
        """Sampling direction: y' and log|det dy'/dy| (FP64)."""
        torch = _native.require_cuda()
        yo = y.clone()
        ld = torch.zeros(y.shape[0], dtype=torch.float64, device=self.dev)
        for l in range(self.layers):
            _native.check(_lib().pbr_flow_layer_forward(self.layer_struct(l), 1, y.shape[0],
                                                        _native.ptr(yo), _native.ptr(ld), None,
                                                        _native.stream_handle()), "flow forward")
        return yo, ld

    def forward_tc(self, y):
        """The sampling direction on the tensor cores: y' and log|det dy'/dy| (FP64) of the
        BF16 network (the weights are converted on every call, so they follow training)."""
        torch = _native.require_cuda()
        assert self.sample_tc, "a layer shape the tensor-core form does not hold"
        lib = _lib()
        p = _native.ptr
        sh = _native.stream_handle()
        if self._tc_packs is None:
            self._tc_packs = [torch.empty(n, dtype=torch.uint8, device=self.dev) for n in self._tc_bytes]
        yo = y.clone()
        ld = torch.zeros(y.shape[0], dtype=torch.float64, device=self.dev)
        st = torch.zeros(1, dtype=torch.int32, device=self.dev)
        for l in range(self.layers):
            layer = self.layer_struct(l)
            _native.check(lib.pbr_flow_tc_pack(layer, p(self._tc_packs[l]), sh), "flow tc pack")
            _native.check(lib.pbr_flow_tc_forward(layer, p(self._tc_packs[l]), y.shape[0], p(yo), p(ld), p(st), sh),
                          "flow tc forward")
        self._tc_status = st
        return yo, ld

    def inverse(self, y, saves=None):
        torch = _native.require_cuda()
        yo = y.clone()
        ld = torch.zeros(y.shape[0], dtype=torch.float64, device=self.dev)
        for l in range(self.layers - 1, -1, -1):
            sv = saves[l] if saves is not None else None
            _native.check(_lib().pbr_flow_layer_forward(self.layer_struct(l), -1, y.shape[0],
                                                        _native.ptr(yo), _native.ptr(ld),
                                                        sv.struct if sv else None,
                                                        _native.stream_handle()), "flow inverse")
        return yo, ld

    def sampling_plan(self):
        """A copy of the rho plan whose source CDF is pi (the learned surface weights)."""
        torch = _native.require_cuda()
        import ctypes
        pi = torch.softmax(torch.as_tensor(self.log_w, dtype=torch.float64, device=self.dev)
                           + self.nu.double(), dim=0)
        Ar = self.prep.A_rho
        cdf = torch.ones(Ar, dtype=torch.float32 if self.plan.precision == 32 else torch.float64,
                         device=self.dev)
        cdf[:self.A] = torch.cumsum(pi, 0).to(cdf.dtype)
        m = _native.PbrModel()
        ctypes.pointer(m)[0] = self.plan.struct
        m.src_cdf = cdf.data_ptr()
        self._cdf = cdf
        return m

    def log_pi_abs(self):
        """ln C_a - ln w_a + ln pi_a: rho's absolute mixture weights with the learned pi."""
        torch = _native.require_cuda()
        return (torch.as_tensor(self.log_k, dtype=torch.float32, device=self.dev) + self.log_pi()).contiguous()

    def sample_and_evaluate(self, X, seed, offset=0, keep=False, tc=None):
        """Draw X proposal samples and evaluate them: returns CUDA tensors s_q (proposal density in
        the scale of g's outputs), s_g, s_gp, s_gm, and with keep also x, y(x).  tc (default: every
        layer's shape allows it) moves the samples with the tensor-core layers."""
        torch = _native.require_cuda()
        from .pimc import evaluate_device
        lib = _lib()
        p = _native.ptr
        q = torch.empty((X, self.N, self.P), dtype=torch.float32, device=self.dev)
        m = self.sampling_plan()
        _native.check(lib.pbr_sample_q(m, int(seed), int(offset), X, p(q), None, _native.stream_handle()),
                      "sample_q")
        y, U = self.prepare(q)
        use_tc = self.sample_tc if tc is None else tc
        yn, logdet = self.forward_tc(y) if use_tc else self.forward(y)
        lse = torch.empty(X, dtype=torch.float64, device=self.dev)
        lpa = self.log_pi_abs()
        _native.check(lib.pbr_flow_base(p(y), None, X, self.D, self.A, p(self.t_mu), p(lpa), None, None,
                                        None, None, p(lse), _native.stream_handle()), "flow base")
        x = torch.empty_like(q)
        _native.check(lib.pbr_flow_apply(p(q), p(y), p(yn), X, self.N, self.P, self.nsel, p(self.t_sigma),
                                         p(x), _native.stream_handle()), "flow apply")
        out = evaluate_device(self.plan, X, q=x)
        s_q = torch.empty(X, dtype=torch.float64, device=self.dev)
        _native.check(lib.pbr_flow_weights(p(lse), p(U), p(logdet), p(out["log_scale"]), X, p(s_q),
                                           _native.stream_handle()), "flow weights")
        status = torch.maximum(out["status"], self._tc_status) if use_tc else out["status"]
        res = {"s_q": s_q, "s_g": out["s_g"], "s_gp": out.get("s_gp"), "s_gm": out.get("s_gm"),
               "status": status}
        if keep:
            res["x"] = x
            res["y"] = self.prepare(x)[0]
        return res

    # ------------------------------------------------------------------------------------------
    @property
    def step_count(self):
        return int(self._step.item())

    def train(self, y, r, epochs=4, batch=8192, lr=1e-3, seed=0, log=None, graph=True):
        """Adam on the weighted forward KL over the dataset (y [X, D] CUDA FP32, r [X] weights).
        A step (minibatch gather, inverse pass, back-propagation, gradients, Adam) runs on fixed
        buffers; with graph=True it is captured as a CUDA graph after its first, eager run and
        replayed for every further minibatch (the step is launch-bound: some 60 launches)."""
        torch = _native.require_cuda()
        X = y.shape[0]
        gen = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        step = None
        for ep in range(epochs):
            perm = torch.randperm(X, generator=gen).to(self.dev)
            tot = torch.zeros((), dtype=torch.float64, device=self.dev)
            for b0 in range(0, X - batch + 1, batch):
                if step is None:
                    step = _TrainStep(self, y, r, batch, lr, graph)
                tot += step(perm[b0:b0 + batch])
            hist.append(float(tot.item()) / max(1, X // batch))
            if log:
                log(f"epoch {ep}: mean batch loss {hist[-1]:.6f}")
        return hist

    def _ensure_buffers(self, B):
        torch = _native.require_cuda()
        if getattr(self, "_bufB", None) == B:
            return
        f32 = dict(dtype=torch.float32, device=self.dev)
        self._saves = []
        for l in range(self.layers):
            I, J = int(self.idx[l][0].numel()), int(self.idx[l][1].numel())
            self._saves.append(_Save(torch, B, I, J, self.H, self.dev))
        Jmax = max(int(b.numel()) for _, b in self.idx)
        self._g_o = torch.empty((B, 2 * Jmax), **f32)
        self._g_z2 = torch.empty((B, self.H), **f32)
        self._g_z1 = torch.empty((B, self.H), **f32)
        lib = _lib()
        n = max(lib.pbr_gemm_tn_scratch(B, m, n) for m, n in ((self.H, 2 * Jmax), (self.H, self.H),
                                                               (max(self.D, 1), self.H)))
        self._scratch = torch.empty(int(n), **f32)
        self._bufB = B

    def gradients(self, y, r):
        """Loss and gradients of one minibatch: inverse pass with saved activations, base loss,
        back-propagation through the layers, weight-gradient GEMMs and bias sums.  Returns
        (loss, [per-layer dict of gradients], gradient of nu); the gradients are views into the
        flat gradient buffer, overwritten by the next call."""
        torch = _native.require_cuda()
        lib = _lib()
        p = _native.ptr
        sh = _native.stream_handle()
        B = y.shape[0]
        self._ensure_buffers(B)
        rt = (r / r.sum()).to(torch.float32).contiguous()
        y0, ld = self.inverse(y, saves=self._saves)
        gy = torch.empty_like(y0)
        rgam = torch.empty((B, self.A), dtype=torch.float32, device=self.dev)
        lterm = torch.empty(B, dtype=torch.float64, device=self.dev)
        lp = self.log_pi().contiguous()
        _native.check(lib.pbr_flow_base(p(y0), p(ld), B, self.D, self.A, p(self.t_mu), p(lp), p(rt),
                                        p(gy), p(rgam), p(lterm), None, sh), "flow base")
        grads = [None] * self.layers
        for l in range(self.layers):                       # the inverse pass ran L-1 .. 0
            st = self.layer_struct(l)
            I, J = st.I, st.J
            g_o = self._g_o if 2 * J == self._g_o.shape[1] else \
                torch.empty((B, 2 * J), dtype=torch.float32, device=self.dev)
            sv = self._saves[l]
            _native.check(lib.pbr_flow_layer_backward(st, B, p(gy), p(rt), sv.struct, p(g_o),
                                                      p(self._g_z2), p(self._g_z1), sh), "flow backward")
            g = self._views(self._gflat, l)
            # weight gradients, with the bias gradient (the column sums of the same B) alongside
            for (A_, B_, M, N, key, bkey) in ((sv.h2, g_o, self.H, 2 * J, "W3", "b3"),
                                              (sv.h1, self._g_z2, self.H, self.H, "W2", "b2"),
                                              (sv.ya, self._g_z1, I, self.H, "W1", "b1")):
                _native.check(lib.pbr_gemm_tn_acc(p(A_), p(B_), B, M, N, 0.0, p(g[key]), p(g[bkey]),
                                                  p(self._scratch), sh), "weight gradient")
            grads[l] = g
        gsum = torch.empty(self.A, dtype=torch.float32, device=self.dev)
        _native.check(lib.pbr_colsum(p(rgam), B, self.A, p(gsum), sh), "nu gradient")
        g_nu = self._gflat[self._nu_off:self._nu_off + self.A]
        torch.neg(gsum - torch.exp(lp) * rt.sum(), out=g_nu)
        return lterm.sum(), grads, g_nu

    def train_step(self, y, r, lr):
        """One Adam step; returns the batch loss as a device scalar (no host synchronisation)."""
        loss, grads, g_nu = self.gradients(y, r)
        self._adam_step(grads, g_nu, lr)
        return loss

    def _adam_step(self, grads, g_nu, lr):
        """One Adam update of every parameter and nu: the gradients are already in the flat
        gradient buffer (grads and g_nu are views into it)."""
        torch = _native.require_cuda()
        lib = _lib()
        p = _native.ptr
        if self._adam is None:
            self._adam = (torch.zeros_like(self._flat), torch.zeros_like(self._flat))
        m, s = self._adam
        _native.check(lib.pbr_adam(p(self._flat), p(self._gflat), p(m), p(s), self._flat.numel(), lr, 0.9, 0.999,
                                   1e-8, p(self._step), _native.stream_handle()), "adam")


class _TrainStep:
    """One training step on fixed buffers (minibatch indices in, batch loss out); after its first
    eager run it is captured as a CUDA graph (graph=True) and replayed."""

    def __init__(self, fl, y, r, batch, lr, graph):
        torch = _native.require_cuda()
        self.fl, self.y, self.r, self.lr, self.want_graph = fl, y, r, lr, graph
        self.idx = torch.empty(batch, dtype=torch.int64, device=fl.dev)
        self.yb = torch.empty((batch,) + tuple(y.shape[1:]), dtype=y.dtype, device=fl.dev)
        self.rb = torch.empty(batch, dtype=r.dtype, device=fl.dev)
        self.loss = torch.zeros((), dtype=torch.float64, device=fl.dev)
        self.graph = None

    def _body(self):
        torch = _native.require_cuda()
        torch.index_select(self.y, 0, self.idx, out=self.yb)
        torch.index_select(self.r, 0, self.idx, out=self.rb)
        self.loss.copy_(self.fl.train_step(self.yb, self.rb, self.lr))

    def __call__(self, idx):
        torch = _native.require_cuda()
        self.idx.copy_(idx)
        if self.graph is not None:
            self.graph.replay()
            return self.loss
        self._body()
        if self.want_graph:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._body()
            self.graph = g
        return self.loss


class _Save:
    def __init__(self, torch, B, I, J, H, dev):
        f32 = dict(dtype=torch.float32, device=dev)
        self.ya = torch.empty((B, I), **f32)
        self.h1 = torch.empty((B, H), **f32)
        self.h2 = torch.empty((B, H), **f32)
        self.s = torch.empty((B, J), **f32)
        self.yb = torch.empty((B, J), **f32)
        st = _native.PbrFlowSave()
        st.ya, st.h1, st.h2, st.s, st.yb = (self.ya.data_ptr(), self.h1.data_ptr(), self.h2.data_ptr(),
                                            self.s.data_ptr(), self.yb.data_ptr())
        self.struct = st
