"""Reverso two-reservoir magma model (models/reverso/reverso/Reverso.py:21-416).

Parameter sets, by name as in the reference: ``Qin`` (basal inflow rate), ``H_s``,
``H_d`` (reservoir depths), ``a_s``, ``a_d`` (reservoir radii) and ``a_c`` (radius
of the hydraulic pipe), one value each.  Material constants as the reference's
properties: ``v`` (Poisson ratio), ``mu`` (viscosity), ``drho`` (density contrast),
``G`` (shear modulus), ``g`` (gravity).

Inputs: a case directory with ``displacements.csv`` in the reference schema
(Data.py: oid, t, x, y, uE, uN, uZ, σE, σN, σZ, the σ columns holding variances),
or the arrays ``txy`` (n x 3), ``d`` (n x 3) and ``var`` (n x 3).  The data
covariance is the diagonal of the variances (Reverso.py:94-106) and the
normalisation -1/2 (log(2π)·n + log det Cd) counts n observation records, as the
reference does (Reverso.py:292-305).

``mode``: "fast" (the reference's default, its C++ forward model: u_E = u_r cos φ)
or "analytic" (its Python strategy: u_E = u_r sin φ, Native.py:96-100); both run
the same FP64 kernel (ag_reverso_llk) with the matching convention.
"""
import csv
import ctypes
import math
import os

import numpy as np
import torch

from .. import _native
from ..device import DEVICE, ptr, require_cuda, stream_handle
from .bayesian import Bayesian

PSETS = ("Qin", "H_s", "H_d", "a_s", "a_d", "a_c")


def read_displacements(path):
    """(txy, d, var) arrays from a displacements.csv in the reference schema."""
    txy, d, var = [], [], []
    with open(path, newline="") as f:
        for rec in csv.DictReader(f):
            txy.append([float(rec["t"]), float(rec["x"]), float(rec["y"])])
            d.append([float(rec["uE"]), float(rec["uN"]), float(rec["uZ"])])
            var.append([float(rec["σE"]), float(rec["σN"]), float(rec["σZ"])])
    return np.array(txy), np.array(d), np.array(var)


def write_displacements(path, txy, d, var, oid=0):
    """Write observations in the reference schema (the synthetic generator's output format)."""
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["oid", "t", "x", "y", "uE", "uN", "uZ", "σE", "σN", "σZ"])
        for p, u, s in zip(txy, d, var):
            w.writerow([oid, *map(repr, map(float, p)), *map(repr, map(float, u)), *map(repr, map(float, s))])


class Reverso(Bayesian):
    def __init__(self, psets, case=None, displacements="displacements.csv", txy=None, d=None, var=None,
                 mode="fast", v=0.25, mu=2000.0, drho=300.0, G=20.0e9, g=9.81, **kwds):
        super().__init__(psets=psets, **kwds)
        if mode not in ("fast", "analytic"):
            raise ValueError(f"mode must be 'fast' or 'analytic' (got {mode!r})")
        if case is not None:
            txy, d, var = read_displacements(os.path.join(case, displacements))
        if txy is None or d is None or var is None:
            raise ValueError("Reverso needs observations: a case directory or the txy, d, var arrays")
        self.txy = np.asarray(txy, dtype=np.float64).reshape(-1, 3)
        self.d = np.asarray(d, dtype=np.float64).reshape(-1, 3)
        self.var = np.asarray(var, dtype=np.float64).reshape(-1, 3)
        if not (len(self.txy) == len(self.d) == len(self.var)):
            raise ValueError("txy, d and var must describe the same observation points")
        if np.any(self.var <= 0.0):
            raise ValueError("variances must be positive")
        self.mode = mode
        self.v, self.mu, self.drho, self.G, self.g = float(v), float(mu), float(drho), float(G), float(g)
        self.observations = len(self.txy)
        self.normalization = -0.5 * (math.log(2.0 * math.pi) * self.observations + float(np.sum(np.log(self.var))))
        self.model = None
        self.strategy = None

    def initialize(self, application):
        super().initialize(application)
        require_cuda()
        missing = [name for name in PSETS if name not in self.psets]
        if missing:
            raise ValueError(f"Reverso needs the parameter sets {PSETS}; missing {missing}")
        self.initializeParameterSets()
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEVICE)
        self._txy, self._d, self._w = dev(self.txy), dev(self.d), dev(1.0 / self.var)
        idx = [self.psets[name].offset for name in PSETS]
        self.model = _native.ReversoModel(self._txy.data_ptr(), self._d.data_ptr(), self._w.data_ptr(),
                                          self.observations, self.parameters, *idx, int(self.mode == "fast"), 0,
                                          self.G, self.v, self.mu, self.drho, self.g)
        self.strategy = self
        return self

    # the strategy interface used by the samplers
    def forward(self, theta, out, mask=None, status=None, residuals=None, stream=None):
        """Data log-likelihood of the rows of theta into out; residuals (optional) receives the
        predicted displacements (n x 3 n_obs, FP64)."""
        _native.call("ag_reverso_llk", ctypes.byref(self.model), ptr(theta), theta.shape[0], self.normalization,
                     ptr(mask), ptr(out), ptr(residuals), stream_handle(stream))
        return out

    def displacements(self, theta, stream=None):
        """Predicted displacements (n x n_obs x 3) of device samples theta."""
        n = theta.shape[0]
        pred = torch.empty(n, 3 * self.observations, dtype=torch.float64, device=DEVICE)
        out = torch.empty(n, dtype=torch.float64, device=DEVICE)
        self.forward(theta, out, residuals=pred, stream=stream)
        return pred.view(n, self.observations, 3)

    def dataLikelihood(self, step):
        self.forward(step.theta, step.data)
        return self
