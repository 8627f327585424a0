"""The CDM oracle against the reference's golden vectors (CPU)."""
import numpy as np
import pytest

from oracle import cdm, cref

G = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "cdm_golden.npz"))


def test_matlab_goldens():
    """Matlab vectors of models/cdm/tests/libcdm.py:27-46 (tolerance of that test, :83-86)."""
    ue, un, uv = cdm.cdm(G["matlab_X"], G["matlab_Y"], *G["matlab_src"])
    for got, key in ((ue, "matlab_ue"), (un, "matlab_un"), (uv, "matlab_uv")):
        ref = G[key]
        assert np.max(np.abs((got - ref) / ref)) < 1e-6


def test_reference_libcdm_outputs():
    """Outputs of the reference models/cdm/cdm/libcdm.py for 24 prior sources."""
    for src, u in zip(G["ref_src"], G["ref_u"]):
        got = np.stack(cdm.cdm(G["ref_X"], G["ref_Y"], *src))
        assert np.max(np.abs(got - u)) <= 1e-10 * np.max(np.abs(u))


def test_c_restatement_matches_numpy():
    lay = cref.RefLayout(10, 0, 2, 9, 3, 6, 0, 0.25)
    X, Y = G["ref_X"], G["ref_Y"]
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    for src, u in zip(G["ref_src"][:6], G["ref_u"][:6]):
        th = np.array(src[:10])
        out, bad = cref.cdm_los(th, lay, X, Y, los)
        assert not bad
        ref = u[0] * 0.38 - u[1] * 0.08 + u[2] * 0.92
        assert np.max(np.abs(out - ref)) <= 1e-10 * np.max(np.abs(ref))


def test_above_surface_raises():
    with pytest.raises(cdm.AboveSurfaceError):
        cdm.cdm(np.zeros(1), np.zeros(1), 0, 0, 500.0, 1000.0, 1000.0, 1000.0, 0, 0, 0, 1.0, 0.25)
    lay = cref.RefLayout(10, 0, 2, 9, 3, 6, 0, 0.25)
    th = np.array([0, 0, 500.0, 1000.0, 1000.0, 1000.0, 0, 0, 0, 1.0])
    _, bad = cref.cdm_los(th, lay, np.zeros(1), np.zeros(1), np.array([[0, 0, 1.0]]))
    assert bad


def test_single_rectangle_cases():
    """A zero semi-axis keeps only the rectangle normal to it (libcdm.py:226-235)."""
    X = np.linspace(-5e3, 5e3, 7)
    Y = np.linspace(-4e3, 4e3, 7)
    v = cdm.vertices(0, 0, 3e3, 0.0, 800.0, 600.0, 10, 20, 30)
    ref = cdm.rectangle(X, Y, v[0], 1.0, 0.25)
    got = cdm.cdm(X, Y, 0, 0, 3e3, 0.0, 800.0, 600.0, 10, 20, 30, 1.0, 0.25)
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-15)
    z = cdm.cdm(X, Y, 0, 0, 3e3, 0.0, 0.0, 0.0, 10, 20, 30, 1.0, 0.25)
    assert all(np.all(c == 0) for c in z)
