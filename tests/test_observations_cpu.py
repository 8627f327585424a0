"""Input readers (no GPU): displacements.csv and cd.txt as the reference's CDM model
reads them (models/cdm/cdm/Data.py:22-39, CDM.py:96-110, 275-355)."""
import csv
import math

import numpy as np
import pytest

from altar_gb300.models.observations import Observations


def write_case(path, x, y, d, theta, phi, cd, oid=None):
    with open(path / "displacements.csv", "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["oid", "x", "y", "d", "theta", "phi"])
        for k in range(len(x)):
            w.writerow([0 if oid is None else int(oid[k]), repr(float(x[k])), repr(float(y[k])),
                        repr(float(d[k])), repr(float(theta[k])), repr(float(phi[k]))])
    np.savetxt(path / "cd.txt", cd, fmt="%.17g")


def _case(rng, m):
    x, y = rng.uniform(-2e4, 2e4, m), rng.uniform(-2e4, 2e4, m)
    theta, phi = rng.uniform(0.2, 0.8, m), rng.uniform(-np.pi, np.pi, m)
    d = rng.normal(0, 1e-2, m)
    return x, y, d, theta, phi


def test_reader_los_and_diagonal_cd(tmp_path):
    """A diagonal cd.txt gives the fused misfit's weights; LOS = (sin θ cos φ, sin θ sin φ, cos θ)."""
    rng = np.random.default_rng(1)
    m = 37
    x, y, d, theta, phi = _case(rng, m)
    var = rng.uniform(1e-5, 4e-5, m)
    write_case(tmp_path, x, y, d, theta, phi, np.diag(var))
    obs = Observations.read(str(tmp_path))
    assert not obs.dense and obs.observations == m and obs.oid is None
    np.testing.assert_array_equal(obs.x, x)
    np.testing.assert_array_equal(obs.d, d)
    np.testing.assert_array_equal(obs.variance, var)
    los = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], 1)
    np.testing.assert_allclose(obs.los, los, rtol=0, atol=1e-15)
    ref = -0.5 * (m * math.log(2 * math.pi) + np.sum(np.log(var)))
    assert abs(obs.normalization() - ref) <= 1e-12 * abs(ref)


def test_reader_dense_cd(tmp_path):
    """A cd.txt with off-diagonal entries is kept dense for the whitening path; the
    normalisation is -1/2 (M log 2π + log det Cd), as the reference computes it from an LU
    (CDM.py:326-339)."""
    rng = np.random.default_rng(2)
    m = 60
    x, y, d, theta, phi = _case(rng, m)
    dist = np.hypot(x[:, None] - x[None, :], y[:, None] - y[None, :])
    cd = 1e-4 * np.exp(-dist / 2e3) + 1e-8 * np.eye(m)
    oid = (x > 0).astype(int)
    write_case(tmp_path, x, y, d, theta, phi, cd, oid=oid)
    obs = Observations.read(str(tmp_path))
    assert obs.dense and obs.cd.shape == (m, m)
    np.testing.assert_array_equal(obs.cd, cd)
    np.testing.assert_array_equal(obs.oid, oid)
    np.testing.assert_array_equal(obs.variance, np.diag(cd))
    sign, logdet = np.linalg.slogdet(cd)
    ref = -0.5 * (m * math.log(2 * math.pi) + logdet)
    assert sign > 0 and abs(obs.normalization() - ref) <= 1e-10 * abs(ref)


def test_reader_rejects_a_wrong_cd_shape(tmp_path):
    rng = np.random.default_rng(3)
    x, y, d, theta, phi = _case(rng, 5)
    write_case(tmp_path, x, y, d, theta, phi, np.eye(4))
    with pytest.raises(ValueError):
        Observations.read(str(tmp_path))
