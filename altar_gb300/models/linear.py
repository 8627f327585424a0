"""Linear Gaussian model d = G θ (models/linear/linear/Linear.py:19-360).

Inputs: Green functions G (M x P), observations d (M) and a dense data
covariance Cd (M x M), given as arrays or read from a case directory with the
reference file names (green.txt, data.txt, cd.txt; Linear.py loadInputs).
Initialisation factors Cd = L Lᵀ once in FP64 and folds it into A = L⁻¹ G,
b = L⁻¹ d; the data log-likelihood
    norm - 1/2 |A θ - b|²,   norm = -1/2 (M log 2π + log det Cd)
is evaluated by ag_linear_llk on the tensor cores (or ag_linear_llk_fp64).
The reference computes norm - |L r|/2 with L = chol(Cd⁻¹) (Linear.py:182); the
two agree only after squaring the norm and only for diagonal Cd.
"""
import ctypes
import math
import os

import numpy as np
import scipy.linalg
import torch

from .. import _native
from ..device import DEVICE, ptr, require_cuda, stream_handle, workspace
from .bayesian import Bayesian


class Linear(Bayesian):
    def __init__(self, psets, green=None, data=None, cd=None, case=None, tensor_cores=True, **kwds):
        super().__init__(psets=psets, **kwds)
        if case is not None:
            green = np.loadtxt(os.path.join(case, "green.txt"), ndmin=2)
            data = np.loadtxt(os.path.join(case, "data.txt"))
            cd = np.loadtxt(os.path.join(case, "cd.txt"), ndmin=2)
        self.G = np.asarray(green, dtype=np.float64)
        self.d = np.asarray(data, dtype=np.float64).ravel()
        self.Cd = np.asarray(cd, dtype=np.float64)
        self.tensor_cores = bool(tensor_cores)
        self.observations = self.d.size
        self._ws = None
        self._ws_bytes = 0
        self.flags = None

    def initialize(self, application):
        super().initialize(application)
        require_cuda()
        self.initializeParameterSets()
        M, P = self.G.shape
        if P != self.parameters or self.d.size != M or self.Cd.shape != (M, M):
            raise ValueError("Green functions, data, covariance and parameter sets disagree in shape")
        L = scipy.linalg.cholesky(self.Cd, lower=True)
        A = scipy.linalg.solve_triangular(L, self.G, lower=True)
        b = scipy.linalg.solve_triangular(L, self.d, lower=True)
        self.normalization = -0.5 * (M * math.log(2.0 * math.pi) + 2.0 * float(np.sum(np.log(np.diag(L)))))
        self.A = torch.from_numpy(np.ascontiguousarray(A)).to(DEVICE)
        self.b = torch.from_numpy(b).to(DEVICE)
        kp = _native.load().ag_linear_kpad(P)
        self.a_split = torch.empty(M * 3 * kp, dtype=torch.int16, device=DEVICE)
        _native.call("ag_linear_prepare", ptr(self.A), M, P, ptr(self.a_split), stream_handle())
        self.model = _native.LinearModel(self.A.data_ptr(), self.b.data_ptr(), self.a_split.data_ptr(), M, P)
        self.flags = torch.zeros(1, dtype=torch.int32, device=DEVICE)
        self.strategy = self
        self.reserve(application.job.chains)
        return self

    def reserve(self, n):
        need = _native.load().ag_linear_workspace_bytes(self.observations, self.parameters, n)
        if need > self._ws_bytes:
            self._ws, self._ws_bytes = workspace(need), need
        return self

    # the strategy interface used by the samplers
    def forward(self, theta, out, mask=None, status=None, residuals=None, stream=None):
        n = theta.shape[0]
        s = stream_handle(stream)
        if self.tensor_cores:
            self.reserve(n)
            _native.call("ag_linear_llk", ctypes.byref(self.model), ptr(theta), n, self.normalization, ptr(out),
                         ptr(self._ws), self._ws_bytes, ptr(self.flags), s)
        else:
            _native.call("ag_linear_llk_fp64", ctypes.byref(self.model), ptr(theta), n, self.normalization,
                         ptr(out), s)
        return out

    def dataLikelihood(self, step):
        self.forward(step.theta, step.data)
        return self
