"""Shared builders for the GPU tests: synthetic problems and a bare model shim."""
import numpy as np
import torch

from altar_gb300 import _native
from altar_gb300.models.forward import CUDA
from altar_gb300.models.observations import Observations
from oracle import cdm

LOS = np.array([0.38, -0.08, 0.92])
CDM_LAYOUT = {"x": 0, "depth": 2, "opening": 3, "ax": 4, "omega": 7}


def cdm_prior_rows(n, seed, reject_above=True):
    """Sources drawn from the CDM workload priors; row = x, y, depth, opening, ax, ay, az, ωx, ωy, ωz."""
    rng = np.random.default_rng(seed)
    rows = []
    while len(rows) < n:
        th = np.array([*rng.uniform(-1e4, 1e4, 2), rng.uniform(1e3, 1e4), rng.uniform(-50, 50),
                       *rng.uniform(100, 3000, 3), *rng.uniform(-90, 90, 3)])
        if reject_above and cdm.above_surface(th[0], th[1], th[2], *th[4:7], *th[7:10]):
            continue
        rows.append(th)
    return np.array(rows)


def min_vertical_angle(th):
    """Smallest angle (degrees) between a rectangle side and the vertical."""
    V = cdm.vertices(th[0], th[1], th[2], *th[4:7], *th[7:10])
    m = 90.0
    for k in range(3):
        for i in range(4):
            s = V[k][(i + 1) % 4] - V[k][i]
            b = np.degrees(np.arccos(-s[2] / np.linalg.norm(s)))
            m = min(m, b, 180.0 - b)
    return m


def cdm_los_oracle(theta, X, Y, los):
    return np.array([cdm.los_displacements(t, CDM_LAYOUT, X, Y, los, 0.25) for t in theta])


class Shim:
    """A minimal model object for the CUDA strategy (observations + layout)."""

    def __init__(self, obs, layout):
        self.obs = obs
        self._layout = layout

    def layout(self):
        return self._layout


def cdm_strategy(X, Y, los, d, var, oid=None, offset_idx=-1, nparams=10, variant=0):
    obs = Observations(X, Y, los, d, var, oid)
    lay = _native.Layout(nparams, 0, 2, 3, 4, 7, offset_idx, 0, 1, 0, variant=variant, nu=0.25)
    return CUDA(_native.AG_MODEL_CDM).initialize(None, Shim(obs, lay)), obs


def mogi_strategy(X, Y, los, d, var, log_strength=False, oid=None, offset_idx=-1, nparams=4,
                  nsources=1, stride=0):
    obs = Observations(X, Y, los, d, var, oid)
    lay = _native.Layout(nparams, 0, 2, 3, -1, -1, offset_idx, int(log_strength), nsources, stride, nu=0.25)
    return CUDA(_native.AG_MODEL_MOGI).initialize(None, Shim(obs, lay)), obs


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype).cuda()
