"""Mogi point sources against several datasets with dense data covariances.

The batched two-source Mogi workload: LOS datasets of uneven sizes, each with
its own dense Cd.  One fused launch of the Mogi kernel evaluates every chain
against the concatenated stations and writes the residual rows; each
dataset's block is then whitened by W = L⁻¹ (Cd = L Lᵀ) on the tensor cores
(ag_whiten_llk).  The log-likelihood is the Gaussian
    -1/2 Σ_k (M_k log 2π + log det Cd_k + r_kᵀ Cd_k⁻¹ r_k).
Parameter sets per source s: ``location{s}`` (2), ``depth{s}`` (1),
``source{s}`` (1), laid out with a constant stride between sources.
"""
import ctypes
import math

import numpy as np
import torch

from .. import _native
from ..device import DEVICE, Stations, ptr, require_cuda, stream_handle, workspace
from .bayesian import Bayesian


class DenseMogi(Bayesian):
    def __init__(self, psets, datasets, nu=0.25, log_strength=True, sources=2, **kwds):
        super().__init__(psets=psets, **kwds)
        self.datasets = datasets
        self.nu = float(nu)
        self.log_strength = bool(log_strength)
        self.sources = int(sources)
        self.kind = _native.AG_MODEL_MOGI
        self._ws = self._resid = None
        self._ws_bytes = 0
        self.strategy = self

    def layout(self):
        p = self.psets
        x0 = p["location0"].offset
        stride = p["location1"].offset - x0 if self.sources > 1 else 0
        for s in range(1, self.sources):
            for name in ("location", "depth", "source"):
                if p[f"{name}{s}"].offset - p[f"{name}0"].offset != s * stride:
                    raise ValueError("multi-source parameter sets need a constant stride between sources")
        return _native.Layout(self.parameters, x0, p["depth0"].offset, p["source0"].offset, -1, -1, -1,
                              int(self.log_strength), self.sources, stride, nu=self.nu)

    def initialize(self, application):
        super().initialize(application)
        require_cuda()
        self.initializeParameterSets()
        xs, ys, los, ds = [], [], [], []
        self.blocks, self._w = [], []
        logdet, col = 0.0, 0
        lib = _native.load()
        for k, ds_k in enumerate(self.datasets):
            m = len(ds_k["x"])
            xs.append(np.asarray(ds_k["x"], float)); ys.append(np.asarray(ds_k["y"], float))
            l = np.asarray(ds_k["los"], float).reshape(-1, 3)
            los.append(np.repeat(l, m, 0) if l.shape[0] == 1 else l)
            ds.append(np.asarray(ds_k["d"], float))
            cd = ds_k["cd"]
            cd = (cd.to(device=DEVICE, dtype=torch.float64) if torch.is_tensor(cd)
                  else torch.as_tensor(np.asarray(cd, float), device=DEVICE))
            L = torch.linalg.cholesky(cd)
            W = torch.linalg.solve_triangular(L, torch.eye(m, dtype=torch.float64, device=DEVICE), upper=False)
            logdet += 2.0 * float(torch.log(torch.diagonal(L)).sum())
            kp = lib.ag_linear_kpad(m)
            wsplit = torch.empty(m * 3 * kp, dtype=torch.int16, device=DEVICE)
            W = W.contiguous()
            _native.call("ag_linear_prepare", ptr(W), m, m, ptr(wsplit), stream_handle())
            self._w.append((W, wsplit))
            self.blocks.append(_native.WhitenBlock(W.data_ptr(), wsplit.data_ptr(), col, m))
            col += m
        self.observations = col
        x, y = np.concatenate(xs), np.concatenate(ys)
        # weights 0: the fused kernel only produces residual rows; the misfit comes from the whitening
        self.stations = Stations(x, y, np.concatenate(los), np.concatenate(ds), np.zeros(col))
        self.normalization = -0.5 * (col * math.log(2.0 * math.pi) + logdet)
        self.layout_struct = self.layout()
        self.flags = torch.zeros(1, dtype=torch.int32, device=DEVICE)
        self.reserve(application.job.chains)
        return self

    def reserve(self, n):
        lib = _native.load()
        need = max(lib.ag_whiten_workspace_bytes(b.m, n) for b in self.blocks)
        if need > self._ws_bytes:
            self._ws, self._ws_bytes = workspace(need), need
        if self._resid is None or self._resid.shape[0] < n:
            self._resid = torch.zeros(n, self.stations.m_padded, dtype=torch.float32, device=DEVICE)
        return self

    def forward(self, theta, out, mask=None, status=None, residuals=None, stream=None):
        n = theta.shape[0]
        self.reserve(n)
        s = stream_handle(stream)
        resid = self._resid[:n]
        _native.call("ag_forward_llk", self.kind, ctypes.byref(self.layout_struct), ptr(theta), n,
                     self.stations.struct, self.normalization, ptr(mask), ptr(out), ptr(status), ptr(resid),
                     None, 0, s)
        for b in self.blocks:
            _native.call("ag_whiten_llk", ctypes.byref(b), ptr(resid), self.stations.m_padded, n, ptr(out),
                         ptr(self._ws), self._ws_bytes, ptr(self.flags), s)
        if residuals is not None:
            residuals.copy_(resid)
        return out

    def dataLikelihood(self, step):
        self.forward(step.theta, step.data)
        return self
