"""Observation inputs of the Mogi and CDM models.

File readers follow the reference schema: ``displacements.csv`` with columns
oid, x, y, d, theta, phi (models/cdm/cdm/Data.py:22-39; LOS from the angles as
in models/cdm/cdm/CDM.py:104-110) and a dense ``cd.txt`` data covariance
(CDM.py:303-321).  A diagonal Cd goes to the fused device misfit (weights
1/σ²); any other Cd is kept dense and the strategies whiten the residuals with
W = L⁻¹ (Cd = L Lᵀ) on the tensor cores.  The log-likelihood is the Gaussian
-1/2 (M log 2π + log det Cd + rᵀ Cd⁻¹ r); the reference's normalisation is the
same (CDM.py:326-339) but its norm ‖chol(Cd⁻¹) r‖ equals rᵀ Cd⁻¹ r only for a
diagonal Cd (altar/altar/norms/L2.py:48-52).
"""
import csv
import math
import os

import numpy as np


class Observations:
    def __init__(self, x, y, los, d, variance=None, oid=None, covariance=None):
        self.x = np.asarray(x, dtype=np.float64)
        self.y = np.asarray(y, dtype=np.float64)
        m = self.x.size
        self.los = np.asarray(los, dtype=np.float64).reshape(-1, 3)
        if self.los.shape[0] == 1:
            self.los = np.repeat(self.los, m, axis=0)
        self.d = np.asarray(d, dtype=np.float64)
        self.cd = None
        if covariance is not None:
            cd = np.asarray(covariance, dtype=np.float64)
            if cd.shape != (m, m):
                raise ValueError(f"data covariance must be {m}x{m}, got {cd.shape}")
            if np.count_nonzero(cd - np.diag(np.diag(cd))):
                self.cd = cd
            variance = np.diag(cd).copy()
        if variance is None:
            raise ValueError("give the data variances or a covariance matrix")
        v = np.asarray(variance, dtype=np.float64)
        self.variance = np.full(m, float(v)) if v.ndim == 0 else v
        self.oid = None if oid is None else np.asarray(oid, dtype=np.int32)
        if not (self.y.size == m and self.los.shape[0] == m and self.d.size == m
                and self.variance.size == m):
            raise ValueError("observation arrays disagree in length")
        if np.any(self.variance <= 0):
            raise ValueError("data variances must be positive")

    @property
    def observations(self):
        return self.x.size

    @property
    def dense(self):
        """True when the data covariance has off-diagonal entries."""
        return self.cd is not None

    @classmethod
    def read(cls, case, displacements="displacements.csv", covariance="cd.txt"):
        rows = []
        with open(os.path.join(case, displacements), newline="") as f:
            for rec in csv.DictReader(f):
                rows.append((int(rec["oid"]), float(rec["x"]), float(rec["y"]), float(rec["d"]),
                             float(rec["theta"]), float(rec["phi"])))
        a = np.array(rows, dtype=np.float64)
        theta, phi = a[:, 4], a[:, 5]
        los = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], 1)
        cd = np.loadtxt(os.path.join(case, covariance), ndmin=2)
        if cd.shape != (len(rows), len(rows)):
            raise ValueError(f"{covariance}: expected {len(rows)}x{len(rows)}, got {cd.shape}")
        oid = a[:, 0].astype(np.int32)
        return cls(a[:, 1], a[:, 2], los, a[:, 3], oid=oid if np.any(oid) else None, covariance=cd)

    def logdet(self):
        """log det Cd (Cholesky for a dense Cd; the reference takes it from an LU, CDM.py:326-339)."""
        if self.cd is None:
            return float(np.sum(np.log(self.variance)))
        L = np.linalg.cholesky(self.cd)
        return 2.0 * float(np.sum(np.log(np.diag(L))))

    def normalization(self):
        return -0.5 * (self.observations * math.log(2.0 * math.pi) + self.logdet())
