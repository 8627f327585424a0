"""CUDA strategy of the point-source models (models/cdm/cdm/CUDA.py:19-107,
models/mogi/mogi/CUDA.py).

Holds the device-resident stations and the parameter layout, and evaluates
the fused forward model + misfit + log-likelihood for a batch of samples.
With a dense data covariance the fused kernel writes the residual rows
instead (station weights 0) and ag_whiten_llk adds -1/2 ‖L⁻¹ r‖² (Cd = L Lᵀ)
on the tensor cores.
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
        self._whiten = None                 # dense Cd: (W, split W, block struct)
        self._wws = None
        self._wws_bytes = 0
        self._resid = None
        self._flags = None

    def initialize(self, application, model):
        require_cuda()
        obs = model.obs
        dense = getattr(obs, "dense", False)
        weight = np.zeros(obs.observations) if dense else 1.0 / obs.variance
        # the CDM stores its stations along a Hilbert curve (compact tiles, fewer quadrature
        # nodes); residual rows keep the caller's order.  Dense Cd whitens residual rows in
        # place, which wants them written in order: no reordering there.
        reorder = self.kind == _native.AG_MODEL_CDM and not dense
        self.stations = Stations(obs.x, obs.y, obs.los, obs.d, weight, obs.oid, reorder=reorder)
        self.layout = model.layout()
        self.norm = obs.normalization()
        if dense:
            self._prepare_whitening(obs.cd)
        self.reserve(application.job.chains if application is not None else 1)
        return self

    def _prepare_whitening(self, cd):
        m = cd.shape[0]
        L = torch.linalg.cholesky(torch.as_tensor(cd, dtype=torch.float64, device=DEVICE))
        W = torch.linalg.solve_triangular(L, torch.eye(m, dtype=torch.float64, device=DEVICE),
                                          upper=False).contiguous()
        kp = _native.load().ag_linear_kpad(m)
        wsplit = torch.empty(m * 3 * kp, dtype=torch.int16, device=DEVICE)
        _native.call("ag_linear_prepare", ptr(W), m, m, ptr(wsplit), stream_handle())
        self._whiten = (W, wsplit, _native.WhitenBlock(W.data_ptr(), wsplit.data_ptr(), 0, m))
        self._flags = torch.zeros(1, dtype=torch.int32, device=DEVICE)

    def reserve(self, n):
        lib = _native.load()
        need = lib.ag_forward_workspace_bytes(self.kind, n)
        if need > self._ws_bytes:
            self._ws = workspace(need)
            self._ws_bytes = need
        if self._whiten is not None:
            wneed = lib.ag_whiten_workspace_bytes(self.stations.m, n)
            if wneed > self._wws_bytes:
                self._wws, self._wws_bytes = workspace(wneed), wneed
            if self._resid is None or self._resid.shape[0] < n:
                self._resid = torch.zeros(n, self.stations.m_padded, dtype=torch.float32, device=DEVICE)
        return self

    @property
    def supports_floor(self):
        """Early rejection: the CDM with diagonal Cd stops a chain's evaluation below its floor."""
        return self.kind == _native.AG_MODEL_CDM and self._whiten is None

    def forward(self, theta, out, mask=None, status=None, residuals=None, stream=None, floor=None):
        """Data log-likelihood of the rows of device θ into device ``out``.  floor (device, one
        value per row, from ag_accept_floor): rows found below it may stop early with -inf."""
        n = theta.shape[0]
        self.reserve(n)
        s = stream_handle(stream)
        resid = residuals
        if self._whiten is not None and resid is None:
            resid = self._resid[:n]
        if floor is not None and resid is None and self.supports_floor:
            _native.call("ag_forward_llk_floor", self.kind, ctypes.byref(self.layout), ptr(theta), n,
                         self.stations.struct, self.norm, ptr(mask), ptr(floor), ptr(out), ptr(status),
                         ptr(self._ws), self._ws_bytes, s)
            return out
        _native.call("ag_forward_llk", self.kind, ctypes.byref(self.layout), ptr(theta), n,
                     self.stations.struct, self.norm, ptr(mask), ptr(out), ptr(status),
                     ptr(resid), ptr(self._ws), self._ws_bytes, s)
        if self._whiten is not None:
            # the fused misfit was 0 (weights 0): add -1/2 ‖W r‖² of the residual rows
            # (rows of masked or rejected chains hold stale values; their llk is not used)
            _native.call("ag_whiten_llk", ctypes.byref(self._whiten[2]), ptr(resid), self.stations.m_padded, n,
                         ptr(out), ptr(self._wws), self._wws_bytes, ptr(self._flags), s)
        return out

    def work(self, theta, stream=None):
        """CDM: FP32 operations (FMA = 2) and special-function operations that the likelihood
        kernel executes for each row of device θ over the m stations, tile by tile (0 above the
        free surface)."""
        n = theta.shape[0]
        flop = torch.empty(n, dtype=torch.float64, device=theta.device)
        sfu = torch.empty(n, dtype=torch.float64, device=theta.device)
        _native.call("ag_cdm_work", ctypes.byref(self.layout), ptr(theta), n, self.stations.struct, ptr(flop),
                     ptr(sfu), stream_handle(stream))
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
