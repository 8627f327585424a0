"""COV annealing schedule (altar/altar/bayesian/COV.py:21-255).

update(step): new β and weights (solver), weighted parameter covariance Σ,
multinomial resampling of the sample by the weights, posterior at the new β.
"""
import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle, workspace
from .grid import Grid


class COV:
    def __init__(self, target=1.0, solver=None):
        self.target = float(target)
        self.solver = solver if solver is not None else Grid()
        self.seed = 0
        self._sigma_ws = None
        self._res_ws = None
        self._alt = None

    def initialize(self, application):
        self.seed = application.rng.seed
        self.solver.initialize(application=application, scheduler=self)
        return self

    def update(self, step):
        self.updateTemperature(step=step)
        self.computeCovariance(step=step)
        theta, (prior, data, posterior) = self.rank(step=step)
        step.theta.copy_(theta)
        step.prior.copy_(prior)
        step.data.copy_(data)
        step.posterior.copy_(posterior)
        return step

    def updateTemperature(self, step):
        return self.solver.solve(step.data, step.state.w, step)

    def computeCovariance(self, step):
        n, p = step.samples, step.parameters
        need = _native.load().ag_sigma_workspace_bytes(n, p)
        if self._sigma_ws is None or self._sigma_ws.numel() < need:
            self._sigma_ws = workspace(need)
        _native.call("ag_weighted_cov", step.state.struct, ptr(step.theta), n, p, ptr(self._sigma_ws),
                     self._sigma_ws.numel(), stream_handle())
        return step.state.sigma

    def rank(self, step, counts=None):
        """Resampled (θ, (prior, data, posterior)) into scratch buffers (COV.py:160-208)."""
        n, p = step.samples, step.parameters
        if self._alt is None or self._alt[0].shape != (n, p):
            f64 = dict(dtype=torch.float64, device=DEVICE)
            self._alt = (torch.zeros(n, p, **f64), torch.zeros(n, **f64), torch.zeros(n, **f64),
                         torch.zeros(n, **f64))
            self._res_ws = workspace(_native.load().ag_resample_workspace_bytes(n))
        th, pr, da, po = self._alt
        _native.call("ag_resample", step.state.struct, n, p, self.seed, ptr(step.theta), ptr(step.prior),
                     ptr(step.data), ptr(th), ptr(pr), ptr(da), ptr(po), ptr(counts),
                     ptr(self._res_ws), self._res_ws.numel(), stream_handle())
        return th, (pr, da, po)
