"""Gaussian misfit norm (altar/altar/norms/L2.py:26-52).

The reference whitens residuals with L = chol(Cd⁻¹) and takes ‖L r‖ (correct
only for diagonal Cd; the correct Gaussian quadratic form is rᵀ Cd⁻¹ r).  The
device path fuses the diagonal case into the forward kernels as
Σ r²/σ²; this class holds the constant part of the log-likelihood.
"""
import math

import numpy as np


class L2:
    @staticmethod
    def normalization(variances):
        """-1/2 (M log 2π + log det Cd) for diagonal Cd (CDM.py:326-339)."""
        v = np.asarray(variances, dtype=np.float64)
        return -0.5 * (v.size * math.log(2.0 * math.pi) + float(np.sum(np.log(v))))
