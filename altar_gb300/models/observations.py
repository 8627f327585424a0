"""Observation inputs of the Mogi and CDM models.

File readers follow the reference schema: ``displacements.csv`` with columns
oid, x, y, d, theta, phi (models/cdm/cdm/Data.py:22-39; LOS from the angles as
in models/cdm/cdm/CDM.py:104-110) and a dense ``cd.txt`` data covariance
(CDM.py:303-321).  The fused device likelihood supports diagonal Cd; a dense
file is accepted when it is diagonal.
"""
import csv
import math
import os

import numpy as np


class Observations:
    def __init__(self, x, y, los, d, variance, oid=None):
        self.x = np.asarray(x, dtype=np.float64)
        self.y = np.asarray(y, dtype=np.float64)
        m = self.x.size
        self.los = np.asarray(los, dtype=np.float64).reshape(-1, 3)
        if self.los.shape[0] == 1:
            self.los = np.repeat(self.los, m, axis=0)
        self.d = np.asarray(d, dtype=np.float64)
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
        diag = np.diag(cd).copy()
        if np.count_nonzero(cd - np.diag(diag)):
            raise NotImplementedError("the fused device likelihood needs a diagonal data covariance")
        oid = a[:, 0].astype(np.int32)
        return cls(a[:, 1], a[:, 2], los, a[:, 3], diag, oid if np.any(oid) else None)

    def normalization(self):
        return -0.5 * (self.observations * math.log(2.0 * math.pi) + float(np.sum(np.log(self.variance))))
