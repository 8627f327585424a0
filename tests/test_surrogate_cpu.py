"""Host-side pieces of the surrogate samplers (no GPU)."""
import numpy as np
import torch

from altar_gb300.bayesian.surrogate import _orthonormal_columns, subset_observations
from altar_gb300.models.observations import Observations


def test_orthonormal_columns():
    """Cholesky QR twice gives an orthonormal basis of the same column space."""
    rng = np.random.default_rng(0)
    Y = torch.from_numpy(rng.normal(size=(500, 12)) @ np.diag(np.logspace(0, 6, 12)))
    Q = _orthonormal_columns(Y.clone())
    np.testing.assert_allclose((Q.T @ Q).numpy(), np.eye(12), atol=1e-10)
    # same span: projecting Y on Q reproduces Y
    P = Q @ (Q.T @ Y)
    assert float(torch.linalg.norm(P - Y) / torch.linalg.norm(Y)) < 1e-10


def test_subset_observations_estimate_the_misfit():
    """Every k-th station with k-fold weights: for a smooth residual field the weighted misfit
    sum of the subset is close to the full one, and the weights scale exactly by k."""
    g = np.linspace(-20e3, 20e3, 200)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    var = np.full(X.size, 9e-6)
    obs = Observations(X, Y, los, np.zeros(X.size), var)
    sub = subset_observations(obs, 16)
    assert sub.x.size == (X.size + 15) // 16
    np.testing.assert_array_equal(sub.x, X[::16])
    np.testing.assert_allclose(sub.variance, var[::16] / 16)
    r = 0.01 * np.exp(-((X - 3e3) ** 2 + (Y + 2e3) ** 2) / (2 * 6e3 ** 2))   # a smooth residual field
    full = np.sum(r * r / var)
    est = np.sum(r[::16] ** 2 / sub.variance)
    assert abs(est - full) < 0.01 * full
