"""Station order for the CDM's per-tile quadrature (altar_gb300/device.py hilbert_order).

The CDM stores its observations along a Hilbert curve so that tiles of 128 consecutive
stations are compact; the likelihood kernel picks each rectangle's quadrature from a
tile's distance, so compact tiles need fewer nodes.  Residual rows are written back in
the caller's order (checked on the GPU against the oracle in test_gpu_forward.py).
"""
import numpy as np

from altar_gb300.device import hilbert_order


def test_curve_on_a_power_of_two_grid():
    """On a 2^k grid the curve visits every point once, each step to a grid neighbour."""
    for k in (1, 2, 3, 5):
        g = np.arange(2 ** k, dtype=float)
        X, Y = [a.ravel() for a in np.meshgrid(g, g)]
        o = hilbert_order(X, Y, bits=k)
        assert sorted(o) == list(range(X.size))
        steps = np.abs(np.diff(X[o])) + np.abs(np.diff(Y[o]))
        assert np.all(steps == 1.0), k


def test_tiles_are_compact_on_the_workload_grid():
    """200 x 200 stations over ±20 km: 128-station tiles in row order span a 25 km row
    segment; along the curve every tile stays within ~5 km."""
    g = np.linspace(-20e3, 20e3, 200)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    o = hilbert_order(X, Y)
    assert sorted(o) == list(range(X.size))
    ext = [max(np.ptp(X[o][t:t + 128]), np.ptp(Y[o][t:t + 128])) for t in range(0, X.size, 128)]
    assert np.median(ext) < 3.5e3 and max(ext) < 5e3
    row = [np.ptp(X[t:t + 128]) for t in range(0, X.size, 128)]
    assert np.median(row) > 20e3


def test_scattered_points_and_duplicates():
    """Any point set: a permutation, stable for repeated points, and a single point."""
    rng = np.random.default_rng(4)
    X, Y = rng.uniform(-3e4, 5e4, 1000), rng.uniform(2e6, 2.01e6, 1000)    # UTM-like offsets
    X[10:20], Y[10:20] = X[5], Y[5]
    o = hilbert_order(X, Y)
    assert sorted(o) == list(range(X.size))
    pos = np.argsort(o)
    dup = np.r_[5, np.arange(10, 20)]
    assert np.all(np.diff(pos[dup]) > 0)       # equal points keep their input order
    assert list(hilbert_order(np.array([1.0]), np.array([2.0]))) == [0]
