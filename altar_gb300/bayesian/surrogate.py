"""Learned surrogate of the forward field and the delayed-acceptance sampler.

No counterpart in the reference.  The surrogate maps source parameters,
normalised by the current population's mean and spread, to K PCA
coefficients of the LOS displacement field:
  * the PCA basis (mean field μ, orthonormal B, per-component scales) comes
    from exact fields of a subset of the current population (randomised range
    finder: B from the leading right singular vectors of the centred fields);
  * training pairs (θ, Bᵀ(u(θ) - μ)/scale) come from those exact evaluations;
  * the network (10 → 4×256 GELU → 64) is trained by the library's own
    forward, backward and Adam kernels (``ag_mlp_*``, ``ag_adam_step``),
    warm-started from the previous stage's weights;
  * its data log-likelihood is evaluated in PCA space (``ag_surrogate_llk``).
A surrogate fitted once over the whole prior is far too coarse for the late,
concentrated populations (measured RMS field error ~4σ on the CDM workload),
so the fit is local to each stage's population and refreshed whenever the
check below fails.

``DelayedAcceptance`` is a Metropolis sampler that, when the surrogate's RMS
field error on held-out chains of the current population is below
``rms_limit`` data standard deviations, screens every proposal on the
surrogate posterior and evaluates the exact model only on the survivors
(Christen & Fox 2005); otherwise it walks exactly like ``Metropolis``.
"""
import ctypes
import math
import time

import numpy as np
import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle, workspace
from .metropolis import Metropolis


def _orthonormal_columns(Y):
    """Orthonormal basis of the columns of a tall FP64 matrix by Cholesky QR, twice
    (Fukaya et al. 2014): the Gram matrices are (k+o) x (k+o) and are factored on the
    host, so no dense solver library runs on the device."""
    for _ in range(2):
        G = (Y.T @ Y).cpu().numpy()
        G += np.eye(G.shape[0]) * (1e-14 * np.trace(G) / G.shape[0] + 1e-300)
        R = np.linalg.cholesky(G).T                                # G = Rᵀ R
        Rinv = np.linalg.solve(R, np.eye(R.shape[0]))
        Y = Y @ torch.from_numpy(Rinv).to(Y.device)
    return Y


class Surrogate:
    def __init__(self, sizes=(10, 256, 256, 256, 256, 64), seed=0, lr=1e-3, batch=4096):
        self.sizes = tuple(int(s) for s in sizes)
        self.k = self.sizes[-1]
        self.net = _native.MLP(len(self.sizes) - 1, (ctypes.c_int32 * 9)(*self.sizes))
        self.seed, self.lr, self.batch = seed, lr, batch
        self.params = self.pbf = self.m = self.v = self.grads = None
        # the tensor-core forward (prediction) needs layer widths that are multiples of 64
        self.tc = all(s % 64 == 0 for s in self.sizes[1:])
        self.wpack = None
        self._tc_flags = None
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
        self.pack()
        return self

    def set_params(self, flat):
        self.params.copy_(torch.as_tensor(flat, dtype=torch.float32))
        _native.call("ag_to_bf16", self.params.numel(), ptr(self.params), ptr(self.pbf), stream_handle())
        self.pack()

    def pack(self):
        """Weights of the tensor-core forward ([W | W] per layer) from the BF16 copy; the buffer
        keeps its device address, so captured graphs that predict stay valid."""
        if not self.tc:
            return self
        lib = _native.load()
        net = ctypes.byref(self.net)
        if self.wpack is None:
            self.wpack = workspace(lib.ag_mlp_tc_pack_bytes(net))
            self._tc_flags = torch.zeros(1, dtype=torch.int32, device=DEVICE)
        _native.call("ag_mlp_tc_pack", net, ptr(self.pbf), ptr(self.wpack), stream_handle())
        return self

    # ---- PCA basis of the LOS fields
    def fit_basis(self, fields, weight, d, norm, oversample=8):
        """Local PCA of exact fields (S, Mp) by a randomised range finder (set-up GEMMs).

        The basis tensors keep their device addresses across refits, so captured
        graphs that read them stay valid.
        """
        F = fields.to(torch.float32)
        mu = F.mean(0)
        Fc = F - mu
        k = min(self.k, F.shape[0] - 1)
        gen = torch.Generator(device=DEVICE)
        gen.manual_seed(self.seed + 7)
        omega = torch.randn(F.shape[1], k + oversample, device=DEVICE, generator=gen)
        Q = _orthonormal_columns((Fc @ omega).double())            # (S, k+o) range of the fields
        Bt = (Q.float().T @ Fc).double()                           # (k+o, Mp)
        # the small (k+o) x (k+o) eigenproblem on the host
        evals, evecs = np.linalg.eigh((Bt @ Bt.T).cpu().numpy())
        order = np.argsort(evals)[::-1][:k]
        lam = torch.from_numpy(np.maximum(evals[order], 1e-30).copy()).to(DEVICE)
        V = torch.from_numpy(np.ascontiguousarray(evecs[:, order])).to(DEVICE)
        B = (Bt.T @ V) / torch.sqrt(lam)                           # orthonormal columns (Mp, k)
        # one common scale (the leading component's spread): the training loss in
        # normalised coefficients is then proportional to the field-space error, so
        # noise-level components cannot dominate it
        scale = torch.full_like(lam, float(torch.sqrt(lam[0] / F.shape[0]).clamp_min(1e-12)))
        if k < self.k:                                             # pad unused components
            B = torch.cat([B, torch.zeros(B.shape[0], self.k - k, dtype=B.dtype, device=DEVICE)], 1)
            scale = torch.cat([scale, torch.ones(self.k - k, dtype=scale.dtype, device=DEVICE)])
        w = weight.to(torch.float64)
        dd = d.to(torch.float64)
        mu64 = mu.double()
        G = B.T @ (w[:, None] * B)
        h = B.T @ (w * (dd - mu64))
        q0 = float(((mu64 - dd) ** 2 * w).sum())
        new = dict(mu=mu, B=B.float(), scale=scale.float(), G=G.float(), h=h.float())
        if self.basis is None:
            self.basis = {key: v.clone() for key, v in new.items()}
        else:
            for key, v in new.items():
                self.basis[key].copy_(v)
        self.basis.update(q0=q0, norm=float(norm))
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
        self.pack()
        return self.losses

    # ---- inference
    needs_fit = True

    def predict(self, theta, lo, hi, out_llk, bufs, mask=None):
        """Surrogate data log-likelihood of device θ rows into out_llk (mask: unused)."""
        n, p = theta.shape
        x, coeff, acts = bufs[0], bufs[1], bufs[2]
        s = stream_handle()
        b = self.basis
        _native.call("ag_normalize_inputs", ptr(theta), n, p, ptr(lo), ptr(hi), ptr(x), s)
        if self.tc:
            # tcgen05 layers (split-BF16 activations, FP32 accumulation); no activations kept
            ws = bufs[3]
            _native.call("ag_mlp_forward_tc", ctypes.byref(self.net), ptr(self.params), ptr(self.wpack), ptr(x),
                         n, ptr(coeff), None, ptr(ws), ws.numel(), ptr(self._tc_flags), s)
        else:
            _native.call("ag_mlp_forward", ctypes.byref(self.net), ptr(self.params), ptr(self.pbf), ptr(x), n,
                         ptr(coeff), ptr(acts), s)
        _native.call("ag_surrogate_llk", n, self.k, ptr(coeff), ptr(b["scale"]), ptr(b["G"]), ptr(b["h"]),
                     b["q0"], b["norm"], ptr(out_llk), s)
        return out_llk

    def buffers(self, n, p):
        lib = _native.load()
        net = ctypes.byref(self.net)
        return (torch.empty(n, p, dtype=torch.float32, device=DEVICE),
                torch.empty(n, self.k, dtype=torch.float32, device=DEVICE),
                torch.empty(lib.ag_mlp_activation_floats(net, n), dtype=torch.float32, device=DEVICE),
                workspace(lib.ag_mlp_tc_workspace_bytes(net, n)) if self.tc else None)

    def reconstruct(self, coeff_norm):
        b = self.basis
        return b["mu"] + (coeff_norm * b["scale"]) @ b["B"].T


class _SubsetModel:
    """The parameter layout of a model over a subset of its observations."""

    def __init__(self, model, obs):
        self.obs = obs
        self._model = model

    def layout(self):
        return self._model.layout()


def subset_observations(obs, k):
    """Every k-th observation of obs with its variance divided by k (its misfit weight
    multiplied by k), so that the subset's misfit sum estimates the full one."""
    from ..models.observations import Observations
    return Observations(obs.x[::k], obs.y[::k], obs.los[::k], obs.d[::k], obs.variance[::k] / k,
                        None if obs.oid is None else obs.oid[::k])


class SubsetSurrogate:
    """Coarse likelihood: the exact forward model on every ``stride``-th observation, with
    the misfit weights multiplied by ``stride``, so that its data log-likelihood estimates
    the full one as a quadrature of the residual field (Christen & Fox 2005 use such a
    coarse model as the first stage of delayed acceptance).  For a smooth displacement
    field the error of a log-likelihood ratio between nearby samples is far below that of
    a fitted network, and nothing is trained; each evaluation costs ~1/stride of the exact
    one.  ``strides`` (coarsest first) are the levels the sampler may pick from, per stage:
    the coarsest whose tempered-ratio check passes.  Works with the point-source models
    whose strategy is the CUDA forward model (CDM, Mogi)."""

    needs_fit = False
    trained = True

    def __init__(self, strides=(32, 16, 8), inner=None):
        """inner: surrogate moves per exact correction at each level (None: the sampler's own
        count at every level); finer levels cost more per move and can take fewer."""
        self.strides = tuple(int(s) for s in (strides if hasattr(strides, "__iter__") else (strides,)))
        self.inner = None if inner is None else tuple(int(k) for k in inner)
        if self.inner is not None and len(self.inner) != len(self.strides):
            raise ValueError("one inner count per stride")
        self.levels = len(self.strides)
        self.level = 0
        self.strategies = []

    @property
    def stride(self):
        return self.strides[self.level]

    def attach(self, application, model):
        from ..models.forward import CUDA
        if not isinstance(getattr(model, "strategy", None), CUDA) or getattr(model, "obs", None) is None:
            raise TypeError("SubsetSurrogate needs a point-source model with station observations (CDM, Mogi)")
        self.strategies = []
        for k in self.strides:
            sub = subset_observations(model.obs, k)
            strat = CUDA(model.strategy.kind).initialize(application=application, model=_SubsetModel(model, sub))
            strat.norm = model.strategy.norm           # constants cancel; keep the exact model's
            self.strategies.append(strat)
        self._main = model.strategy
        return self

    def predict(self, theta, lo, hi, out_llk, bufs, mask=None, floor=None):
        """Coarse data log-likelihood of device θ rows into out_llk; rows flagged in mask are
        skipped and sources above the surface are flagged there; with floor (early rejection
        of the first-stage moves) rows found below it may stop with -inf."""
        strat = self.strategies[self.level]
        strat.layout.variant = self._main.layout.variant   # the exact model's (autotuned) launch shape
        strat.forward(theta, out_llk, mask=mask, status=mask, floor=floor)
        return out_llk

    @property
    def supports_floor(self):
        return bool(self.strategies) and getattr(self.strategies[self.level], "supports_floor", False)

    def buffers(self, n, p):
        return None


class DelayedAcceptance(Metropolis):
    """Metropolis with a surrogate screen (stage 1) before the exact model (stage 2)."""

    # the walk changes with per-stage host decisions; it does not shard
    static_walk = False
    shardable = False

    def __init__(self, surrogate=None, rms_limit=0.5, delta_limit=2.0, fit_chains=4096, check_chains=256,
                 epochs=40, refit_epochs=None, start_beta=0.0, stop_beta=0.1, retry_every=3, spread=3.0,
                 inner=10, outer=1, screen_limit=None, screen_steps=None, **kwds):
        """rms_limit: largest RMS field error (data standard deviations) of a usable surrogate;
        delta_limit: largest spread (standard deviation over trial proposals) of the error of
        the surrogate's tempered log-posterior ratio, β[(s(y) - s(x)) - (l(y) - l(x))].  Delayed
        acceptance stays exact whatever the surrogate, but its mixing needs the surrogate's
        accept decisions to follow the exact ones: with 40,000 observations a field error far
        below the noise can still move the log-likelihood ratio by tens of units near β = 1.
        inner: surrogate Metropolis moves per exact correction (1 = two-stage delayed
        acceptance; k > 1 = surrogate-transition proposals, Liu 2001, corrected by the same
        exact second stage); outer: exact corrections per stage in the surrogate mode
        (None: the job's steps).  start_beta, stop_beta: the surrogate is used only for
        start_beta <= β < stop_beta; the stages after stop_beta walk exactly, which lets
        the final population relax with the exact kernel alone.  The defaults (10 surrogate
        moves and one exact correction per stage, ratio spread up to 2, exact stages from
        β = 0.1) were the fastest setting measured on the CDM workload with the MLP surrogate
        whose posterior summaries matched plain Metropolis to within its own run-to-run
        spread.  With the coarse-model surrogate (SubsetSurrogate) the fastest setting that
        reached the converged posterior on that workload was inner=20, outer=1,
        delta_limit=1.0, stop_beta=1.0."""
        super().__init__(**kwds)
        self.delta_limit = float(delta_limit)
        # coarse-model surrogates: when no level passes delta_limit for the surrogate-transition
        # walk but the finest passes screen_limit, the stage walks with two-stage delayed
        # acceptance (every step screened by the coarse model, the exact model on the survivors)
        self.screen_limit = None if screen_limit is None else float(screen_limit)
        # two-stage steps per screened stage (None: the job's steps); a screened step costs a
        # coarse evaluation plus an exact one for the survivors only, so a screened stage can
        # afford the longer walk that keeps the population mixed
        self.screen_steps = None if screen_steps is None else int(screen_steps)
        self.delta = None
        self._prepare_s = 0.0
        self._backoff = 0
        self.inner = int(inner)
        self.outer = None if outer is None else int(outer)
        self.surrogate = surrogate if surrogate is not None else Surrogate(batch=1024)
        self.rms_limit = float(rms_limit)
        self.fit_chains, self.check_chains = int(fit_chains), int(check_chains)
        self.epochs, self.start_beta, self.stop_beta = int(epochs), float(start_beta), float(stop_beta)
        # later fits start from the previous weights and need fewer passes
        self.refit_epochs = self.epochs if refit_epochs is None else int(refit_epochs)
        self.retry_every, self.spread = int(retry_every), float(spread)
        self.mode = "plain"
        self.rms = None
        self.refits = 0
        self.screened = None
        self._stage = 0
        self._last_try = -10 ** 9
        self._bounds = None
        self._sbufs = None
        self._chain = None

    def initialize(self, application):
        super().initialize(application)
        if not self.surrogate.needs_fit:
            self.surrogate.attach(application, application.model)
        # start the device BLAS the refits use now, so that its one-time set-up does not
        # land inside the first refit
        for dt in (torch.float32, torch.float64):
            a = torch.ones(64, 64, dtype=dt, device=DEVICE)
            (a @ a).sum().item()
        return self

    def mode_key(self):
        # each level of a subset surrogate reads other stations: one captured walk per level
        if self.mode in ("da", "screen") and not self.surrogate.needs_fit:
            return f"{self.mode}{self.surrogate.level}"
        return self.mode

    def report(self):
        rep = {"mode": self.mode, "rms_sigma": self.rms, "delta_sd": self.delta, "refits": self.refits,
               "prepare_s": self._prepare_s}
        if self.mode in ("da", "screen") and self.screened is not None:
            rep["screened"] = int(self.screened.item())
        if self.mode in ("da", "screen") and not self.surrogate.needs_fit:
            rep["stride"] = self.surrogate.stride
        return rep

    # ---- per-stage host decisions (eager, before the walk graph)
    def prepare(self, annealer, step):
        t0 = time.perf_counter()
        try:
            return self._prepare(annealer, step)
        finally:
            self._prepare_s = time.perf_counter() - t0

    def _prepare(self, annealer, step):
        self._stage += 1
        if self.screened is not None:
            self.screened.zero_()
        beta = step.beta
        if beta < self.start_beta or beta >= self.stop_beta:
            self.mode = "plain"
            return self
        model, strat = annealer.model, annealer.model.strategy
        sur = self.surrogate
        n, p = step.samples, step.parameters
        fit = min(self.fit_chains, n // 2)
        chk = min(self.check_chains, n - fit)
        stride = max(1, n // (fit + chk))
        rows = torch.arange(0, n, stride, device=DEVICE)[: fit + chk]
        fit_rows, chk_rows = rows[:fit], rows[fit:fit + chk]
        if not sur.needs_fit:
            # nothing to fit: the coarsest level whose tempered-ratio check passes, else exact
            self._set_bounds(step)
            self.rms = None
            level, self.delta = self._delta_check(annealer, step, chk_rows, levels=range(sur.levels))
            sur.level = level
            self.mode = "da" if self._usable() else "plain"
            if self.mode == "plain" and self.screen_limit is not None and self.delta <= self.screen_limit:
                self.mode = "screen"
            return self
        if sur.trained:
            self.rms = self._check(annealer, step, chk_rows)
            self.delta = self._delta_check(annealer, step, chk_rows)
            if self._usable():
                self.mode = "da"
                return self
            # after a fit that failed its own check, wait retry_every stages before fitting again
            if self._backoff and self._stage - self._last_try < self.retry_every:
                self.mode = "plain"
                return self
        self._last_try = self._stage
        self._refit(annealer, step, fit_rows)
        self.rms = self._check(annealer, step, chk_rows)
        self.delta = self._delta_check(annealer, step, chk_rows)
        self._backoff = 0 if self._usable() else 1
        self.mode = "da" if self._usable() else "plain"
        return self

    def _usable(self):
        return (self.rms is None or self.rms <= self.rms_limit) and self.delta <= self.delta_limit

    def _delta_check(self, annealer, step, rows, levels=None):
        """Spread of β[(s(y) - s(x)) - (l(y) - l(x))] over one trial proposal per check chain.
        levels: surrogate levels to try in order (SubsetSurrogate); returns the first level
        whose spread is within delta_limit together with its spread, else the last one's."""
        model, strat, sur = annealer.model, annealer.model.strategy, self.surrogate
        th = step.theta.index_select(0, rows).contiguous()
        ex_x = step.data.index_select(0, rows)
        c, p = th.shape
        f64 = dict(dtype=torch.float64, device=DEVICE)
        cand, cprior = torch.empty(c, p, **f64), torch.empty(c, **f64)
        mask = torch.zeros(c, dtype=torch.int32, device=DEVICE)
        s = stream_handle()
        st = step.state.struct
        _native.call("ag_cholesky_scaled", st, p, s)
        _native.call("ag_propose", st, ptr(th), c, p, ptr(model.lo), ptr(model.hi), self.seed, 900000 + self._stage,
                     ptr(cand), ptr(mask), ptr(cprior), s)
        ex_y = torch.empty(c, **f64)
        strat.forward(cand, ex_y, mask=mask, status=mask)
        bufs = sur.buffers(c, p)
        sx, sy = torch.empty(c, **f64), torch.empty(c, **f64)
        ok = mask == 0
        result = (None, float("inf"))
        for level in (levels if levels is not None else [None]):
            if level is not None:
                sur.level = level
            sur.predict(th, self._bounds[0], self._bounds[1], sx, bufs)
            sur.predict(cand, self._bounds[0], self._bounds[1], sy, bufs)
            if int(ok.sum()) < 2:
                return (level, float("inf")) if levels is not None else float("inf")
            eps = step.beta * ((sy - sx) - (ex_y - ex_x))[ok]
            result = (level, float(eps.std()))
            if result[1] <= self.delta_limit:
                break
        return result if levels is not None else result[1]

    def _fields(self, strat, theta):
        n = theta.shape[0]
        res = torch.zeros(n, strat.stations.m_padded, dtype=torch.float32, device=DEVICE)
        out = torch.empty(n, dtype=torch.float64, device=DEVICE)
        strat.forward(theta, out, residuals=res)
        return res + strat.stations.data_rows

    def _set_bounds(self, step):
        th = step.theta
        mean = th.mean(0)
        sd = th.std(0)
        width = torch.maximum(self.spread * sd, 1e-9 * (mean.abs() + 1.0))
        lo, hi = mean - width, mean + width
        if self._bounds is None:
            self._bounds = (lo.clone(), hi.clone())
        else:
            self._bounds[0].copy_(lo)
            self._bounds[1].copy_(hi)

    def _refit(self, annealer, step, rows):
        model, strat, sur = annealer.model, annealer.model.strategy, self.surrogate
        th = step.theta.index_select(0, rows).contiguous()
        self._set_bounds(step)
        fields = self._fields(strat, th)
        sur.fit_basis(fields, strat.stations.weight_rows, strat.stations.data_rows, strat.norm)
        p = step.parameters
        x = torch.empty(th.shape[0], p, dtype=torch.float32, device=DEVICE)
        _native.call("ag_normalize_inputs", ptr(th), th.shape[0], p, ptr(self._bounds[0]), ptr(self._bounds[1]),
                     ptr(x), stream_handle())
        if sur.params is None:
            sur.init_params()
        sur.reserve(th.shape[0], p)
        sur.add(x, sur.coefficients(fields))
        sur.train(epochs=self.epochs if self.refits == 0 else self.refit_epochs)
        self.refits += 1

    def _check(self, annealer, step, rows):
        """RMS of surrogate minus exact LOS field over stations, in data standard deviations."""
        strat, sur = annealer.model.strategy, self.surrogate
        th = step.theta.index_select(0, rows).contiguous()
        exact = self._fields(strat, th)
        bufs = sur.buffers(th.shape[0], th.shape[1])
        tmp = torch.empty(th.shape[0], dtype=torch.float64, device=DEVICE)
        sur.predict(th, self._bounds[0], self._bounds[1], tmp, bufs)
        approx = sur.reconstruct(bufs[1])
        w = strat.stations.weight_rows
        err2 = ((approx - exact) ** 2 * w).sum(1) / strat.stations.m
        return float(torch.sqrt(err2.mean()))

    def _inner(self):
        """Surrogate moves per exact correction: the surrogate's per-level count if it has one."""
        per_level = getattr(self.surrogate, "inner", None)
        return int(per_level[self.surrogate.level]) if per_level else self.inner

    # ---- walks
    def walkChains(self, annealer, step):
        if self.mode == "da":
            if self.inner > 1:
                return self._walk_transition(annealer, step)
            return self._walk_da(annealer, step)
        if self.mode == "screen":
            return self._walk_da(annealer, step)
        return super().walkChains(annealer, step)

    def _walk_transition(self, annealer, step):
        """k surrogate Metropolis moves, then one exact correction of where they ended."""
        model = annealer.model
        strat = model.strategy
        sur = self.surrogate
        n, p = step.samples, step.parameters
        cand, cprior, cdata, mask = self._buffers(n, p)
        if self._sbufs is None or self._sbufs[1].shape[0] != n:
            self._sbufs = (sur.buffers(n, p), torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int64, device=DEVICE))
        if self._chain is None or self._chain[0].shape != (n, p):
            f64 = dict(dtype=torch.float64, device=DEVICE)
            st = step.state
            counters = torch.zeros(3, dtype=torch.int64, device=DEVICE)
            sst = _native.StageState(*(t.data_ptr() for t in (st.beta, st.dbeta_cov, st.scaling, st.sigma,
                                                             st.chol, st.w, counters, st.epoch, st.flags)))
            self._chain = (torch.zeros(n, p, **f64), torch.zeros(n, **f64), torch.zeros(n, **f64),
                           torch.zeros(n, **f64), torch.zeros(n, dtype=torch.int32, device=DEVICE), sst, counters,
                           torch.empty(n, **f64))
        bufs, sur_cur, sur_cand, passed, index, count, screened = self._sbufs
        th_s, pr_s, su_s, po_s, mask2, sst, _, floor = self._chain
        # early rejection of the first-stage moves (the coarse model's Metropolis test)
        early = self.early_reject and getattr(sur, "supports_floor", False)
        self.screened = screened
        lo, hi = self._bounds
        st = step.state.struct
        s = stream_handle()
        sur.predict(step.theta, lo, hi, sur_cur, bufs)
        outer = self.outer if self.outer is not None else self.steps
        for o in range(outer):
            th_s.copy_(step.theta)
            pr_s.copy_(step.prior)
            su_s.copy_(sur_cur)
            _native.call("ag_posterior", st, n, ptr(pr_s), ptr(su_s), ptr(po_s), s)
            inner = self._inner()
            for j in range(inner):
                sid = 1000 + o * inner + j
                _native.call("ag_propose", st, ptr(th_s), n, p, ptr(model.lo), ptr(model.hi), self.seed, sid,
                             ptr(cand), ptr(mask), ptr(cprior), s)
                if early:
                    _native.call("ag_accept_floor", ctypes.byref(sst), n, self.seed, sid, ptr(mask), ptr(cprior),
                                 ptr(po_s), ptr(floor), s)
                    sur.predict(cand, lo, hi, sur_cand, bufs, mask=mask, floor=floor)
                else:
                    sur.predict(cand, lo, hi, sur_cand, bufs, mask=mask)
                _native.call("ag_accept", ctypes.byref(sst), n, p, self.seed, sid, ptr(mask), ptr(cand),
                             ptr(cprior), ptr(sur_cand), ptr(th_s), ptr(pr_s), ptr(su_s), ptr(po_s), s)
            _native.call("ag_da_moved", n, p, ptr(step.theta), ptr(th_s), ptr(passed), ptr(index), ptr(count), s)
            mask2.zero_()
            if self.early_reject and getattr(strat, "supports_floor", False):
                # early rejection of the exact correction (the stage-2 test's own uniform)
                _native.call("ag_da_floor", st, n, self.seed, o, ptr(mask2), ptr(passed), ptr(pr_s), ptr(su_s),
                             ptr(step.prior), ptr(sur_cur), ptr(step.posterior), ptr(floor), s)
                _native.call("ag_forward_llk_subset_floor", strat.kind, ctypes.byref(strat.layout), ptr(th_s), n,
                             strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(floor), ptr(cdata),
                             ptr(mask2), ptr(strat._ws), strat._ws_bytes, s)
            else:
                _native.call("ag_forward_llk_subset", strat.kind, ctypes.byref(strat.layout), ptr(th_s), n,
                             strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(cdata), ptr(mask2),
                             None, ptr(strat._ws), strat._ws_bytes, s)
            _native.call("ag_da_accept", st, n, p, self.seed, o, ptr(mask2), ptr(passed), ptr(th_s), ptr(pr_s),
                         ptr(cdata), ptr(su_s), ptr(step.theta), ptr(step.prior), ptr(step.data),
                         ptr(step.posterior), ptr(sur_cur), ptr(screened), s)
        return step.state.counters

    def _walk_da(self, annealer, step):
        model = annealer.model
        strat = model.strategy
        sur = self.surrogate
        n, p = step.samples, step.parameters
        cand, cprior, cdata, mask = self._buffers(n, p)
        if self._sbufs is None or self._sbufs[1].shape[0] != n:
            self._sbufs = (sur.buffers(n, p), torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.float64, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.empty(n, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int32, device=DEVICE),
                           torch.zeros(1, dtype=torch.int64, device=DEVICE))
        bufs, sur_cur, sur_cand, passed, index, count, screened = self._sbufs
        self.screened = screened
        lo, hi = self._bounds
        st = step.state.struct
        s = stream_handle()
        early = self.early_reject and getattr(strat, "supports_floor", False)
        if early and (getattr(self, "_dfloor", None) is None or self._dfloor.shape[0] != n):
            self._dfloor = torch.empty(n, dtype=torch.float64, device=DEVICE)
        # the constant parts of the surrogate log-likelihood (q0, norm) cancel in both stages
        sur.predict(step.theta, lo, hi, sur_cur, bufs)
        steps = self.screen_steps if (self.mode == "screen" and self.screen_steps) else self.steps
        for k in range(steps):
            _native.call("ag_propose", st, ptr(step.theta), n, p, ptr(model.lo), ptr(model.hi), self.seed, k,
                         ptr(cand), ptr(mask), ptr(cprior), s)
            sur.predict(cand, lo, hi, sur_cand, bufs, mask=mask)
            _native.call("ag_da_screen", st, n, self.seed, k, ptr(mask), ptr(cprior), ptr(sur_cand),
                         ptr(step.prior), ptr(sur_cur), ptr(passed), ptr(index), ptr(count), s)
            if early:
                # early rejection of the exact stage (the stage-2 test's own uniform)
                _native.call("ag_da_floor", st, n, self.seed, k, ptr(mask), ptr(passed), ptr(cprior), ptr(sur_cand),
                             ptr(step.prior), ptr(sur_cur), ptr(step.posterior), ptr(self._dfloor), s)
                _native.call("ag_forward_llk_subset_floor", strat.kind, ctypes.byref(strat.layout), ptr(cand), n,
                             strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(self._dfloor),
                             ptr(cdata), ptr(mask), ptr(strat._ws), strat._ws_bytes, s)
            else:
                _native.call("ag_forward_llk_subset", strat.kind, ctypes.byref(strat.layout), ptr(cand), n,
                             strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(cdata), ptr(mask),
                             None, ptr(strat._ws), strat._ws_bytes, s)
            _native.call("ag_da_accept", st, n, p, self.seed, k, ptr(mask), ptr(passed), ptr(cand), ptr(cprior),
                         ptr(cdata), ptr(sur_cand), ptr(step.theta), ptr(step.prior), ptr(step.data),
                         ptr(step.posterior), ptr(sur_cur), ptr(screened), s)
        return step.state.counters
