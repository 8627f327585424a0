"""CUDA strategy of the point-source models (models/cdm/cdm/CUDA.py:19-107,
models/mogi/mogi/CUDA.py).

Holds the device-resident stations and the parameter layout, and evaluates
the fused forward model + misfit + log-likelihood for a batch of samples.
Device tensors are used in place; host (numpy) samples are copied in and the
log-likelihoods copied back, which is the reference's call pattern
(host θ in, host data likelihood out).
"""
import ctypes

import numpy as np
import torch

from .. import _native
from ..device import DEVICE, Stations, ptr, require_cuda, stream_handle, workspace


class CUDA:
    def __init__(self, kind):
        self.kind = kind
        self.stations = None
        self.layout = None
        self.norm = 0.0
        self._ws = None
        self._ws_bytes = 0

    def initialize(self, application, model):
        require_cuda()
        obs = model.obs
        self.stations = Stations(obs.x, obs.y, obs.los, obs.d, 1.0 / obs.variance, obs.oid)
        self.layout = model.layout()
        self.norm = obs.normalization()
        self.reserve(application.job.chains if application is not None else 1)
        return self

    def reserve(self, n):
        need = _native.load().ag_forward_workspace_bytes(self.kind, n)
        if need > self._ws_bytes:
            self._ws = workspace(need)
            self._ws_bytes = need
        return self

    def forward(self, theta, out, mask=None, status=None, residuals=None, stream=None):
        """Data log-likelihood of the rows of device θ into device ``out``."""
        n = theta.shape[0]
        self.reserve(n)
        _native.call("ag_forward_llk", self.kind, ctypes.byref(self.layout), ptr(theta), n,
                     self.stations.struct, self.norm, ptr(mask), ptr(out), ptr(status),
                     ptr(residuals), ptr(self._ws), self._ws_bytes, stream_handle(stream))
        return out

    def work(self, theta, stream=None):
        """CDM: FP32 operations (FMA = 2) and special-function operations per station that the
        likelihood kernel executes for each row of device θ (0 above the free surface)."""
        n = theta.shape[0]
        flop = torch.empty(n, dtype=torch.int32, device=theta.device)
        sfu = torch.empty(n, dtype=torch.int32, device=theta.device)
        _native.call("ag_cdm_work", ctypes.byref(self.layout), ptr(theta), n, ptr(flop), ptr(sfu),
                     stream_handle(stream))
        return flop, sfu

    def dataLikelihood(self, model, step):
        theta = step.theta
        if isinstance(theta, np.ndarray):
            # reference call pattern: host samples in, host log-likelihoods out
            th = torch.from_numpy(np.ascontiguousarray(theta, dtype=np.float64)).to(DEVICE, non_blocking=True)
            out = torch.empty(th.shape[0], dtype=torch.float64, device=DEVICE)
            self.forward(th, out)
            step.data[:] = out.cpu().numpy()
            return self
        self.forward(theta, step.data)
        return self
