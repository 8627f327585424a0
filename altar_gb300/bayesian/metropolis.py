"""Metropolis sampler (altar/altar/bayesian/Metropolis.py:21-291).

Same configuration (scaling .1, acceptanceWeight 8, rejectionWeight 1) and
the same per-step semantics: propose θ' = θ + (L z)ᵀ with L = chol(scaling² Σ),
reject samples outside the model's support (and, for the CDM, above the free
surface), evaluate the likelihoods of every candidate, accept where
log u <= post' - post.  Each step is three launches: propose (+verify +prior),
the fused forward model, accept.

early_reject: before the forward model, the log-likelihood below which each proposal is
certainly rejected (the accept test's own uniform, ag_accept_floor); a forward model that
supports it stops evaluating such a candidate part way (Solonen et al. 2012, "Efficient
MCMC for climate model parameter estimation: parallel adaptive chains and early
rejection", Bayesian Analysis 7(3)).  The accept decisions, hence the chains, are the
same as with full evaluations; only work for rejected candidates is saved.
"""
import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle


class Metropolis:
    def __init__(self, scaling=0.1, acceptanceWeight=8.0, rejectionWeight=1.0, early_reject=True):
        self.scaling = float(scaling)
        self.acceptanceWeight = float(acceptanceWeight)
        self.rejectionWeight = float(rejectionWeight)
        self.early_reject = bool(early_reject)
        self.steps = 1
        self.seed = 0
        self._buf = None
        self._floor = None

    def initialize(self, application):
        self.steps = application.job.steps
        self.seed = application.rng.seed
        return self

    def _buffers(self, n, p):
        if self._buf is None or self._buf[0].shape != (n, p):
            f64 = dict(dtype=torch.float64, device=DEVICE)
            self._buf = (torch.zeros(n, p, **f64), torch.zeros(n, **f64), torch.zeros(n, **f64),
                         torch.zeros(n, dtype=torch.int32, device=DEVICE))
        return self._buf

    # hooks of the annealing worker: host-side decisions before a walk, and the
    # key under which the walk's launch sequence is captured
    capturable = True
    # each chain's walk depends on its own row and global index only: a rank can walk a block
    shardable = True
    # the walk's launches are the same every stage: a whole stage can replay as one graph
    static_walk = True

    def prepare(self, annealer, step):
        return self

    def mode_key(self):
        return "mh"

    def report(self):
        return {}

    def prime(self, step):
        """Set the initial proposal scaling on the device."""
        step.state.scaling.fill_(self.scaling)
        return self

    def samplePosterior(self, annealer, step):
        d = annealer.dispatcher
        d.notify(event=d.samplePosteriorStart, controller=annealer)
        self.prepareSamplingPDF(annealer=annealer, step=step)
        stats = self.walkChains(annealer=annealer, step=step)
        d.notify(event=d.samplePosteriorFinish, controller=annealer)
        return stats

    def resample(self, annealer, statistics):
        """Adapt the proposal scaling from the acceptance counters (device)."""
        self.adjustCovarianceScaling(annealer.worker.step)
        return

    def prepareSamplingPDF(self, annealer, step):
        d = annealer.dispatcher
        d.notify(event=d.prepareSamplingPDFStart, controller=annealer)
        _native.call("ag_cholesky_scaled", step.state.struct, step.parameters, stream_handle())
        d.notify(event=d.prepareSamplingPDFFinish, controller=annealer)

    def walkChains(self, annealer, step):
        model = annealer.model
        d = annealer.dispatcher
        n, p = step.samples, step.parameters
        cand, cprior, cdata, mask = self._buffers(n, p)
        st = step.state.struct
        s = stream_handle()
        early = self.early_reject and getattr(model.strategy, "supports_floor", False)
        if early and (self._floor is None or self._floor.shape[0] != n):
            self._floor = torch.empty(n, dtype=torch.float64, device=DEVICE)
        for k in range(self.steps):
            d.notify(event=d.chainAdvanceStart, controller=annealer)
            d.notify(event=d.verifyStart, controller=annealer)
            _native.call("ag_propose", st, ptr(step.theta), n, p, ptr(model.lo), ptr(model.hi),
                         self.seed, k, ptr(cand), ptr(mask), ptr(cprior), s)
            d.notify(event=d.verifyFinish, controller=annealer)
            d.notify(event=d.dataStart, controller=annealer)
            if early:
                _native.call("ag_accept_floor", st, n, self.seed, k, ptr(mask), ptr(cprior), ptr(step.posterior),
                             ptr(self._floor), s)
                model.strategy.forward(cand, cdata, mask=mask, status=mask, floor=self._floor)
            else:
                model.strategy.forward(cand, cdata, mask=mask, status=mask)
            d.notify(event=d.dataFinish, controller=annealer)
            d.notify(event=d.acceptStart, controller=annealer)
            _native.call("ag_accept", st, n, p, self.seed, k, ptr(mask), ptr(cand), ptr(cprior),
                         ptr(cdata), ptr(step.theta), ptr(step.prior), ptr(step.data),
                         ptr(step.posterior), s)
            d.notify(event=d.acceptFinish, controller=annealer)
            d.notify(event=d.chainAdvanceFinish, controller=annealer)
        # accepted, rejected, unlikely stay on the device until the stage report
        return step.state.counters

    def adjustCovarianceScaling(self, step):
        _native.call("ag_adapt_scaling", step.state.struct, self.acceptanceWeight,
                     self.rejectionWeight, stream_handle())
        return self
