"""State of the calculation at one β (altar/altar/bayesian/CoolingStep.py:17-180).

All arrays live on the GPU: θ (samples x parameters, FP64), the prior, data
and posterior log-likelihoods, and Σ.  β and the sampler's per-stage scalars
live in a small device block (``StageState``) so that the stage kernels, and
CUDA graphs of them, never need the host.
"""
import copy
import ctypes

import torch

from .. import _native
from ..device import DEVICE, ptr


class StageState:
    """Device block behind ``ag_stage_state``."""

    def __init__(self, samples, parameters, chain0=0):
        """chain0: global index of the first row when the population is split across ranks
        (the proposal and accept streams are keyed by the global chain index)."""
        f64 = dict(dtype=torch.float64, device=DEVICE)
        self.scalars = torch.zeros(8, **f64)          # β, δβ, cov, scaling
        self.beta = self.scalars[0:1]
        self.dbeta_cov = self.scalars[1:3]
        self.scaling = self.scalars[3:4]
        self.sigma = torch.zeros(parameters, parameters, **f64)
        self.chol = torch.zeros(parameters, parameters, **f64)
        self.w = torch.zeros(samples, **f64)
        self.counters = torch.zeros(3, dtype=torch.int64, device=DEVICE)
        self.epoch = torch.zeros(1, dtype=torch.int32, device=DEVICE)
        self.flags = torch.zeros(1, dtype=torch.int32, device=DEVICE)
        self.chain0 = int(chain0)
        self._s = self._struct(self.chain0)

    def _struct(self, chain0):
        return _native.StageState(*(t.data_ptr() for t in (
            self.beta, self.dbeta_cov, self.scaling, self.sigma, self.chol, self.w, self.counters,
            self.epoch, self.flags)), chain0, 0)

    def view(self, chain0):
        """The same device block, described to the kernels as starting at global chain chain0."""
        v = copy.copy(self)
        v.chain0 = int(chain0)
        v._s = self._struct(v.chain0)
        return v

    @property
    def struct(self):
        return ctypes.byref(self._s)


class CoolingStep:
    def __init__(self, beta, theta, likelihoods, sigma=None, state=None):
        self.theta = theta
        self.prior, self.data, self.posterior = likelihoods
        n, p = theta.shape
        self.state = state if state is not None else StageState(n, p)
        if sigma is not None:
            self.state.sigma.copy_(sigma)
        self.state.beta.fill_(float(beta))

    @property
    def samples(self):
        return self.theta.shape[0]

    @property
    def parameters(self):
        return self.theta.shape[1]

    @property
    def beta(self):
        return float(self.state.beta.item())

    @beta.setter
    def beta(self, value):
        self.state.beta.fill_(float(value))

    @property
    def sigma(self):
        return self.state.sigma

    @classmethod
    def alloc(cls, samples, parameters):
        f64 = dict(dtype=torch.float64, device=DEVICE)
        theta = torch.zeros(samples, parameters, **f64)
        lk = tuple(torch.zeros(samples, **f64) for _ in range(3))
        return cls(beta=0.0, theta=theta, likelihoods=lk)

    @classmethod
    def start(cls, annealer):
        """Initial sample from the prior and its likelihoods at β = 0 (CoolingStep.py:53-71)."""
        model = annealer.model
        step = cls.alloc(samples=model.job.chains, parameters=model.parameters)
        model.initializeSample(step=step)
        model.likelihoods(annealer=annealer, step=step)
        return step

    def clone(self):
        st = StageState(self.samples, self.parameters)
        st.scalars.copy_(self.state.scalars)
        st.sigma.copy_(self.state.sigma)
        return CoolingStep(beta=self.beta, theta=self.theta.clone(),
                           likelihoods=(self.prior.clone(), self.data.clone(), self.posterior.clone()),
                           state=st)

    def computePosterior(self):
        """posterior = prior + β data (CoolingStep.py:103-113)."""
        _native.call("ag_posterior", self.state.struct, self.samples, ptr(self.prior), ptr(self.data),
                     ptr(self.posterior), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self

    def print(self, channel=None, indent="  "):
        lines = [f"step", f"{indent}β: {self.beta}",
                 f"{indent}θ: ({self.samples} samples) x ({self.parameters} parameters)"]
        text = "\n".join(lines)
        if channel is not None:
            channel(text)
        return text
