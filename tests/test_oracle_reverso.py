"""Reverso oracle against the reference's own forward model (golden vectors), and the
host side of the Reverso model plugin (no GPU).

tests/golden/reverso_golden.npz holds (u_r, u_z) from the reference's
models/reverso/reverso/libreverso.py (generated by tests/golden/make_reverso_golden.py)
for 16 samples at 75 observation points.
"""
import math
import os

import numpy as np

from altar_gb300.models.reverso import read_displacements, write_displacements
from oracle import reverso

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reverso_golden.npz"))
MATERIAL = dict(zip(("G", "v", "mu", "drho", "g"), (float(x) for x in G["material"])))


def test_oracle_matches_reference_forward_model():
    for th, ur, uz in zip(G["theta"], G["u_r"], G["u_z"]):
        r, z = reverso.radial_vertical(th, G["txy"], **MATERIAL)
        np.testing.assert_allclose(r, ur, rtol=1e-13, atol=1e-15 * np.abs(ur).max())
        np.testing.assert_allclose(z, uz, rtol=1e-13, atol=1e-15 * np.abs(uz).max())


def test_east_north_conventions():
    th, txy = G["theta"][3], G["txy"]
    phi = np.arctan2(txy[:, 2], txy[:, 1])
    fast = reverso.displacements(th, txy, east_cos=True, **MATERIAL)
    analytic = reverso.displacements(th, txy, east_cos=False, **MATERIAL)
    np.testing.assert_allclose(fast[:, 0], G["u_r"][3] * np.cos(phi), rtol=1e-13, atol=1e-18)
    np.testing.assert_allclose(fast[:, 1], G["u_r"][3] * np.sin(phi), rtol=1e-13, atol=1e-18)
    np.testing.assert_array_equal(fast[:, 0], analytic[:, 1])
    np.testing.assert_array_equal(fast[:, 2], analytic[:, 2])


def test_normalization_counts_observation_points():
    """Reverso.py:292-305 multiplies log 2π by the number of records, not of data values."""
    var = np.full((35, 3), 4e-4)
    expect = -0.5 * (35 * math.log(2 * math.pi) + 105 * math.log(4e-4))
    assert abs(reverso.normalization(var) - expect) <= 1e-13 * abs(expect)


def test_displacements_csv_round_trip(tmp_path):
    txy, d, var = reverso.synthetic_case()
    path = str(tmp_path / "displacements.csv")
    write_displacements(path, txy, d, var)
    t2, d2, v2 = read_displacements(path)
    np.testing.assert_array_equal(t2, txy)
    np.testing.assert_array_equal(d2, d)
    np.testing.assert_array_equal(v2, var)
    assert len(txy) == 35 and np.all(var >= 1e-4)
