"""Learned surrogate of the forward field and the delayed-acceptance sampler.

No counterpart in the reference.  The surrogate maps normalised source
parameters to K PCA coefficients of the LOS displacement field:
  * the PCA basis (mean field μ, orthonormal B, per-component scales) comes
    from exact fields the sampler evaluated in its first stages (Gram matrix
    of a subset and its leading eigenvectors, computed once as set-up);
  * training pairs (θ, Bᵀ(u(θ) - μ)/scale) are collected from every exact
    evaluation while β is below ``collect_until_beta`` (up to ``max_samples``);
  * the network (10 → 4×256 GELU → 64) is trained by the library's own
    forward, backward and Adam kernels (``ag_mlp_*``, ``ag_adam_step``);
  * its data log-likelihood is evaluated in PCA space (``ag_surrogate_llk``).

``DelayedAcceptance`` is a Metropolis sampler that, once the surrogate is
trained and its RMS field error on the current population is below
``rms_limit`` data standard deviations, screens every proposal on the
surrogate posterior and evaluates the exact model only on the survivors
(Christen & Fox 2005); otherwise it walks exactly like ``Metropolis``.
"""
import ctypes
import math

import numpy as np
import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle, workspace
from .metropolis import Metropolis


class Surrogate:
    def __init__(self, sizes=(10, 256, 256, 256, 256, 64), seed=0, lr=1e-3, batch=4096):
        self.sizes = tuple(int(s) for s in sizes)
        self.k = self.sizes[-1]
        self.net = _native.MLP(len(self.sizes) - 1, (ctypes.c_int32 * 9)(*self.sizes))
        self.seed, self.lr, self.batch = seed, lr, batch
        self.params = self.pbf = self.m = self.v = self.grads = None
        self.step_count = 0
        self.basis = None
        self.trained = False
        self._x = self._y = None
        self.count = 0
        self.losses = []

    # ---- parameters
    def init_params(self):
        rng = np.random.default_rng(self.seed)
        chunks = []
        for fi, fo in zip(self.sizes[:-1], self.sizes[1:]):
            chunks.append(rng.normal(0.0, math.sqrt(2.0 / fi), fo * fi))
            chunks.append(np.zeros(fo))
        p = np.concatenate(chunks).astype(np.float32)
        assert p.size == _native.load().ag_mlp_param_count(ctypes.byref(self.net))
        self.params = torch.from_numpy(p).to(DEVICE)
        self.pbf = torch.empty(p.size, dtype=torch.int16, device=DEVICE)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        _native.call("ag_to_bf16", p.size, ptr(self.params), ptr(self.pbf), stream_handle())
        self.step_count = 0
        return self

    def set_params(self, flat):
        self.params.copy_(torch.as_tensor(flat, dtype=torch.float32))
        _native.call("ag_to_bf16", self.params.numel(), ptr(self.params), ptr(self.pbf), stream_handle())

    # ---- PCA basis of the LOS fields
    def fit_basis(self, fields, weight, d, norm, sample=4096):
        """fields: (S, Mp) exact LOS fields (padding columns have weight 0)."""
        F = fields[:sample].to(torch.float64)
        mu = F.mean(0)
        Fc = F - mu
        gram = Fc @ Fc.T
        evals, evecs = torch.linalg.eigh(gram)
        idx = torch.argsort(evals, descending=True)[: self.k]
        lam = evals[idx].clamp_min(1e-300)
        B = (Fc.T @ evecs[:, idx]) / torch.sqrt(lam)           # orthonormal columns
        scale = torch.sqrt(lam / F.shape[0])                      # std of each coefficient
        w = weight.to(torch.float64)
        dd = d.to(torch.float64)
        G = B.T @ (w[:, None] * B)
        h = B.T @ (w * (dd - mu))
        q0 = float(((mu - dd) ** 2 * w).sum())
        self.basis = dict(mu=mu.float(), B=B.float(), scale=scale.float(), G=G.float(), h=h.float(), q0=q0,
                          norm=float(norm), explained=float(lam.sum() / evals.clamp_min(0).sum()))
        return self.basis

    def coefficients(self, fields):
        """Normalised PCA coefficients of exact fields (n, Mp) -> (n, K)."""
        b = self.basis
        return ((fields - b["mu"]) @ b["B"]) / b["scale"]

    # ---- training data and training
    def reserve(self, max_samples, p):
        self._x = torch.empty(max_samples, p, dtype=torch.float32, device=DEVICE)
        self._y = torch.empty(max_samples, self.k, dtype=torch.float32, device=DEVICE)
        self.count = 0

    def add(self, x, y):
        n = min(x.shape[0], self._x.shape[0] - self.count)
        if n > 0:
            self._x[self.count:self.count + n] = x[:n]
            self._y[self.count:self.count + n] = y[:n]
            self.count += n
        return n

    @property
    def full(self):
        return self._x is not None and self.count >= self._x.shape[0]

    def train(self, epochs=8, lr=None):
        lib = _native.load()
        lr = self.lr if lr is None else lr
        n_all = self.count
        B = min(self.batch, n_all)
        acts = torch.empty(lib.ag_mlp_activation_floats(ctypes.byref(self.net), B), dtype=torch.float32,
                           device=DEVICE)
        out = torch.empty(B, self.k, dtype=torch.float32, device=DEVICE)
        dout = torch.empty_like(out)
        scratch = torch.empty(2 * B * max(self.sizes), dtype=torch.float32, device=DEVICE)
        rowloss = torch.empty(B, dtype=torch.float32, device=DEVICE)
        gen = torch.Generator(device=DEVICE)
        gen.manual_seed(self.seed)
        s = stream_handle()
        net = ctypes.byref(self.net)
        for ep in range(epochs):
            perm = torch.randperm(n_all, device=DEVICE, generator=gen)
            tot = torch.zeros((), dtype=torch.float64, device=DEVICE)
            for b0 in range(0, n_all - B + 1, B):
                sel = perm[b0:b0 + B]
                xb = self._x.index_select(0, sel)
                yb = self._y.index_select(0, sel)
                _native.call("ag_mlp_forward", net, ptr(self.params), ptr(self.pbf), ptr(xb), B, ptr(out),
                             ptr(acts), s)
                _native.call("ag_mse_grad", B, self.k, ptr(out), ptr(yb), ptr(dout), ptr(rowloss), s)
                _native.call("ag_mlp_backward", net, ptr(self.params), ptr(self.pbf), ptr(xb), B, ptr(acts),
                             ptr(dout), ptr(self.grads), ptr(scratch), s)
                self.step_count += 1
                _native.call("ag_adam_step", self.params.numel(), ptr(self.params), ptr(self.grads), ptr(self.m),
                             ptr(self.v), self.step_count, lr, 0.9, 0.999, 1e-8, ptr(self.pbf), s)
                tot += rowloss.double().mean()
            self.losses.append(float(tot) / max(1, n_all // B))
        self.trained = True
        return self.losses

    # ---- inference
    def predict(self, theta, lo, hi, out_llk, bufs):
        """Surrogate data log-likelihood of device θ rows into out_llk."""
        n, p = theta.shape
        x, coeff, acts = bufs
        s = stream_handle()
        b = self.basis
        _native.call("ag_normalize_inputs", ptr(theta), n, p, ptr(lo), ptr(hi), ptr(x), s)
        _native.call("ag_mlp_forward", ctypes.byref(self.net), ptr(self.params), ptr(self.pbf), ptr(x), n,
                     ptr(coeff), ptr(acts), s)
        _native.call("ag_surrogate_llk", n, self.k, ptr(coeff), ptr(b["scale"]), ptr(b["G"]), ptr(b["h"]),
                     b["q0"], b["norm"], ptr(out_llk), s)
        return out_llk

    def buffers(self, n, p):
        lib = _native.load()
        return (torch.empty(n, p, dtype=torch.float32, device=DEVICE),
                torch.empty(n, self.k, dtype=torch.float32, device=DEVICE),
                torch.empty(lib.ag_mlp_activation_floats(ctypes.byref(self.net), n), dtype=torch.float32,
                            device=DEVICE))

    def reconstruct(self, coeff_norm):
        b = self.basis
        return b["mu"] + (coeff_norm * b["scale"]) @ b["B"].T


class DelayedAcceptance(Metropolis):
    """Metropolis with a surrogate screen (stage 1) before the exact model (stage 2)."""

    def __init__(self, surrogate=None, collect_until_beta=0.05, max_samples=2_000_000, rms_limit=0.5,
                 epochs=8, collect_per_step=8192, **kwds):
        super().__init__(**kwds)
        self.surrogate = surrogate if surrogate is not None else Surrogate()
        self.collect_until_beta = collect_until_beta
        self.max_samples = max_samples
        self.rms_limit = rms_limit
        self.epochs = epochs
        self.collect_per_step = collect_per_step
        self.mode = "collect"
        self.rms_history = []
        self.screened = None
        self._resid = None
        self._sbufs = None

    @property
    def capturable(self):
        return self.mode != "collect"

    def initialize(self, application):
        super().initialize(application)
        return self

    # graphs: the worker keys captured walks by mode
    def mode_key(self):
        return self.mode

    def prepare(self, annealer, step):
        """Host-side decisions before a walk: train when collection ends, check the surrogate."""
        self._choose_mode(annealer, step)
        if self.screened is not None:
            self.screened.zero_()
        return self

    def report(self):
        rep = {"mode": self.mode, "samples": self.surrogate.count}
        if self.rms_history and self.mode != "collect":
            rep["rms_sigma"] = self.rms_history[-1]
        if self.mode == "da" and self.screened is not None:
            rep["screened"] = int(self.screened.item())
        return rep

    def _choose_mode(self, annealer, step):
        sur = self.surrogate
        if self.mode == "collect":
            beta = step.beta
            if (beta >= self.collect_until_beta or sur.full) and sur.count > 0:
                sur.train(epochs=self.epochs)
                self.mode = "da"
            else:
                return
        # per-stage check of the surrogate on the current population
        rms = self.field_rms(annealer, step)
        self.rms_history.append(rms)
        self.mode = "da" if rms <= self.rms_limit else "plain"

    def field_rms(self, annealer, step, count=256):
        """RMS of surrogate minus exact LOS field over stations, in data standard deviations."""
        model = annealer.model
        strat = model.strategy
        th = step.theta[:count].contiguous()
        n = th.shape[0]
        mp = strat.stations.m_padded
        res = torch.zeros(n, mp, dtype=torch.float32, device=DEVICE)
        out = torch.empty(n, dtype=torch.float64, device=DEVICE)
        strat.forward(th, out, residuals=res)
        exact = res + strat.stations.losd[:, 3]
        bufs = self.surrogate.buffers(n, th.shape[1])
        sur_llk = torch.empty(n, dtype=torch.float64, device=DEVICE)
        self.surrogate.predict(th, model.lo, model.hi, sur_llk, bufs)
        approx = self.surrogate.reconstruct(bufs[1])
        w = strat.stations.weight
        m = strat.stations.m
        err2 = ((approx - exact) ** 2 * w).sum(1) / m
        return float(torch.sqrt(err2.mean()))

    def walkChains(self, annealer, step):
        if self.mode == "collect":
            return self._walk_collect(annealer, step)
        if self.mode == "da":
            return self._walk_da(annealer, step)
        return super().walkChains(annealer, step)

    def _walk_collect(self, annealer, step):
        """Exact walk that also records (θ, PCA coefficients) pairs for training."""
        model = annealer.model
        strat = model.strategy
        sur = self.surrogate
        n, p = step.samples, step.parameters
        cand, cprior, cdata, mask = self._buffers(n, p)
        mp = strat.stations.m_padded
        nc = min(n, self.collect_per_step)
        if self._resid is None or self._resid.shape != (nc, mp):
            self._resid = torch.zeros(nc, mp, dtype=torch.float32, device=DEVICE)
        st = step.state.struct
        s = stream_handle()
        dobs = strat.stations.losd[:, 3]
        for k in range(self.steps):
            _native.call("ag_propose", st, ptr(step.theta), n, p, ptr(model.lo), ptr(model.hi), self.seed, k,
                         ptr(cand), ptr(mask), ptr(cprior), s)
            strat.forward(cand, cdata, mask=mask, status=mask)
            # fields of the first nc candidates (a second pass over a slice keeps the buffer small)
            sub = cand[:nc]
            tmp = torch.empty(nc, dtype=torch.float64, device=DEVICE)
            strat.forward(sub, tmp, mask=mask[:nc], residuals=self._resid)
            valid = mask[:nc] == 0
            fields = (self._resid + dobs)[valid]
            if sur.basis is None:
                sur.fit_basis(fields, strat.stations.weight, dobs, strat.norm)
                sur.reserve(self.max_samples, p)
                sur.init_params()
            if not sur.full and fields.shape[0] > 0:
                xb = torch.empty(fields.shape[0], p, dtype=torch.float32, device=DEVICE)
                thv = sub[valid].contiguous()
                _native.call("ag_normalize_inputs", ptr(thv), thv.shape[0], p, ptr(model.lo), ptr(model.hi),
                             ptr(xb), s)
                sur.add(xb, sur.coefficients(fields))
            _native.call("ag_accept", st, n, p, self.seed, k, ptr(mask), ptr(cand), ptr(cprior), ptr(cdata),
                         ptr(step.theta), ptr(step.prior), ptr(step.data), ptr(step.posterior), s)
        return step.state.counters

    def _walk_da(self, annealer, step):
        model = annealer.model
        strat = model.strategy
        sur = self.surrogate
        n, p = step.samples, step.parameters
        cand, cprior, cdata, mask = self._buffers(n, p)
        if self._sbufs is None or self._sbufs[0].shape[0] != n:
            self._sbufs = (sur.buffers(n, p), torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int64, device=DEVICE))
        bufs, sur_cur, sur_cand, passed, index, count, screened = self._sbufs
        self.screened = screened
        st = step.state.struct
        s = stream_handle()
        sur.predict(step.theta, model.lo, model.hi, sur_cur, bufs)
        for k in range(self.steps):
            _native.call("ag_propose", st, ptr(step.theta), n, p, ptr(model.lo), ptr(model.hi), self.seed, k,
                         ptr(cand), ptr(mask), ptr(cprior), s)
            sur.predict(cand, model.lo, model.hi, sur_cand, bufs)
            _native.call("ag_da_screen", st, n, self.seed, k, ptr(mask), ptr(cprior), ptr(sur_cand),
                         ptr(step.prior), ptr(sur_cur), ptr(passed), ptr(index), ptr(count), s)
            strat.reserve(n)
            _native.call("ag_forward_llk_subset", strat.kind, ctypes.byref(strat.layout), ptr(cand), n,
                         strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(cdata), ptr(mask), None,
                         ptr(strat._ws), strat._ws_bytes, s)
            _native.call("ag_da_accept", st, n, p, self.seed, k, ptr(mask), ptr(passed), ptr(cand), ptr(cprior),
                         ptr(cdata), ptr(sur_cand), ptr(step.theta), ptr(step.prior), ptr(step.data),
                         ptr(step.posterior), ptr(sur_cur), ptr(screened), s)
        return step.state.counters
