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


@pytest.mark.parametrize("beta_deg", [10.0, 2.0, 170.0, 178.0])
def test_steep_pair_same_in_both_configurations(beta_deg):
    """The likelihood kernel evaluates a near-vertical side in the ratio configuration
    (β if cos β > 0, β - π otherwise) at every station, where the reference picks the
    configuration by the sign of y1 (libcdm.py:342-362).  The basis: the two
    configurations give the same pair at the free surface except near the singular ray of
    the other one, which the ratio configuration does not have (r - z3 > 0 there)."""
    beta = np.radians(beta_deg)
    sb, cb = np.sin(beta), np.cos(beta)
    aA, L, b = 3000.0, 1000.0, (0.3, -0.7, 0.5)
    g = np.linspace(-8000.0, 8000.0, 17)
    y1, y2 = [a.ravel() for a in np.meshgrid(g + 37.0, g - 11.0)]

    def pair(beff):
        va = cdm.angular_dislocation(y1, y2, beff, *b, 0.25, aA)
        vb = cdm.angular_dislocation(y1 - L * sb, y2, beff, *b, 0.25, aA + L * cb)
        return np.array([vb[i] - va[i] for i in range(3)])

    ratio = pair(beta if cb > 0 else beta - np.pi)
    other = pair(beta - np.pi if cb > 0 else beta)
    scale = np.max(np.abs(ratio))
    # the pair is ~1e-3 of the single dislocations (O(|b|) = O(1)), whose FP64 rounding it
    # inherits times cot²β: agreement means 1e-9 of the pair plus 2e-14 cot²β; a
    # configuration mismatch would be O(1) relative
    assert np.max(np.abs(ratio - other)) <= 1e-9 * scale + 2e-14 * (cb / sb) ** 2
    # r - z3 (z3 = y1 sin β' - a cos β' for the configuration angle β') vanishes on the other
    # configuration's singular ray, which meets the surface at y1 = ±a tan β; for the ratio
    # configuration it stays >= (1 - sin β) r at every surface station
    def r_minus_z3(beff, y1v, y2v):
        r = np.sqrt(y1v * y1v + y2v * y2v + aA * aA)
        return (r - (y1v * np.sin(beff) - aA * np.cos(beff))) / r

    b_ratio, b_other = (beta, beta - np.pi) if cb > 0 else (beta - np.pi, beta)
    y0 = np.array([-aA * np.tan(beta) if cb > 0 else aA * np.tan(np.pi - beta)])
    assert r_minus_z3(b_other, y0, np.zeros(1))[0] < 1e-12
    wide = np.linspace(-50e3, 50e3, 401)
    w1, w2 = [a.ravel() for a in np.meshgrid(wide, wide)]
    assert np.min(r_minus_z3(b_ratio, w1, w2)) >= (1.0 - sb) * (1.0 - 1e-12)
