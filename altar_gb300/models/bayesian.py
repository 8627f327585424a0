"""Base class of Bayesian models (altar/altar/models/Bayesian.py:19-180).

Same hooks as the reference (initialize, posterior, initializeSample,
priorLikelihood, dataLikelihood, posteriorLikelihood, likelihoods, verify,
top, bottom); the sample-wide work runs in the C-ABI kernels on the GPU.
"""
import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle


class Bayesian:
    offset = 0
    parameters = 0

    def __init__(self, psets=None, **kwds):
        self.psets = dict(psets or {})
        self.job = None
        self.rng = None
        self.controller = None
        self.lo = self.hi = self.prep_lo = self.prep_hi = None

    # protocol obligations
    def initialize(self, application):
        self.job = application.job
        self.rng = application.rng
        self.controller = application.controller
        return self

    def posterior(self, application):
        return self.controller.posterior(model=self)

    def initializeParameterSets(self):
        offset = 0
        for name, pset in self.psets.items():
            offset += pset.initialize(model=self, offset=offset)
        self.parameters = offset
        lo, hi, plo, phi = [], [], [], []
        for pset in self.psets.values():
            a, b = pset.prior_bounds()
            c, d = pset.prep_bounds()
            lo += a; hi += b; plo += c; phi += d
        as_dev = lambda v: torch.tensor(v, dtype=torch.float64, device=DEVICE)
        self.lo, self.hi, self.prep_lo, self.prep_hi = as_dev(lo), as_dev(hi), as_dev(plo), as_dev(phi)
        return self

    def meta(self, path="parameters.csv"):
        """Persist the sample layout: one row (name, count, offset) per parameter set, the
        file the reference's models write at initialisation (models/cdm/cdm/CDM.py:358-380)."""
        import csv
        with open(path, mode="w", newline="") as stream:
            writer = csv.writer(stream)
            writer.writerow(["name", "count", "offset"])
            for name, pset in self.psets.items():
                writer.writerow([name, pset.count, pset.offset])
        return self

    def initializeSample(self, step, attempt=0, redraw=None):
        """θ from the prep distributions (Base.py:44-54)."""
        _native.call("ag_prior_sample", step.samples, self.parameters, ptr(self.prep_lo),
                     ptr(self.prep_hi), self.rng.seed, attempt, ptr(redraw), ptr(step.theta),
                     stream_handle())
        return self

    def priorLikelihood(self, step):
        _native.call("ag_prior_llk", ptr(step.theta), step.samples, self.parameters, ptr(self.lo),
                     ptr(self.hi), None, ptr(step.prior), stream_handle())
        return self

    def dataLikelihood(self, step):
        raise NotImplementedError(f"model '{type(self).__name__}' must implement 'dataLikelihood'")

    def posteriorLikelihood(self, step):
        _native.call("ag_posterior", step.state.struct, step.samples, ptr(step.prior),
                     ptr(step.data), ptr(step.posterior), stream_handle())
        return self

    def likelihoods(self, annealer, step):
        dispatcher = annealer.dispatcher
        dispatcher.notify(event=dispatcher.priorStart, controller=annealer)
        self.priorLikelihood(step=step)
        dispatcher.notify(event=dispatcher.priorFinish, controller=annealer)
        dispatcher.notify(event=dispatcher.dataStart, controller=annealer)
        self.dataLikelihood(step=step)
        dispatcher.notify(event=dispatcher.dataFinish, controller=annealer)
        dispatcher.notify(event=dispatcher.posteriorStart, controller=annealer)
        self.posteriorLikelihood(step=step)
        dispatcher.notify(event=dispatcher.posteriorFinish, controller=annealer)
        return self

    def verify(self, step, mask):
        """mask[i] |= out-of-support bit (Uniform.verify, Contiguous.verify)."""
        _native.call("ag_prior_llk", ptr(step.theta), step.samples, self.parameters, ptr(self.lo),
                     ptr(self.hi), ptr(mask), None, stream_handle())
        return mask

    def top(self, step):
        return self

    def bottom(self, step):
        return self

    def restrict(self, theta):
        return theta[:, self.offset:self.offset + self.parameters]
