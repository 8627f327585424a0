"""CATMIP oracle pieces: known answers and self-consistency (CPU)."""
import math

import numpy as np

from oracle import catmip, philox


def test_philox_known_answers():
    """Random123 known-answer vectors for Philox4x32-10."""
    cases = [((0, 0, 0, 0), (0, 0), "6627e8d5 e169c58d bc57ac4c 9b00dbd8"),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), "408f276d 41c83b0e a20bc7c6 6d5451fd"),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
              "d16cfe09 94fdcceb 5001e420 24126ea1")]
    for ctr, key, want in cases:
        r = philox.philox4x32_10(*[np.array([c], dtype=np.uint64) for c in ctr], *key)
        assert " ".join("%08x" % int(x[0]) for x in r) == want


def test_uniform_ranges():
    u = philox.resample_uniforms(7, 100000, 3)
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01
    a = philox.accept_uniforms(7, 100000, 0, 0)
    assert a.min() > 0.0 and a.max() <= 1.0
    z = philox.proposal_normals(7, 50000, 4, 1, 2)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02


def test_mogi_closed_form():
    """Directly above the source the LOS response is (1-ν) ΔV d nz /(π d³)."""
    th = np.array([[0.0, 0.0, 3000.0, 2e6]])
    los = np.array([[0.0, 0.0, 1.0]])
    u = catmip.mogi_los(th, np.array([0.0]), np.array([0.0]), los, 0.25, log_strength=False)
    assert math.isclose(u[0, 0], (1 - 0.25) * 2e6 / (math.pi * 3000.0 ** 2), rel_tol=1e-14)
    # log10 parameterisation of the reference (mogi/Native.py:169)
    u2 = catmip.mogi_los(np.array([[0.0, 0.0, 3000.0, math.log10(2e6)]]), np.array([0.0]),
                         np.array([0.0]), los, 0.25, log_strength=True)
    assert math.isclose(u2[0, 0], u[0, 0], rel_tol=1e-12)


def test_cov_grid_skip_to_one():
    """Nearly equal log-likelihoods: COV stays below target, β jumps to 1 (COV.cc:257-268)."""
    llk = np.linspace(-1.0, -0.999, 1000)
    b, db, cov, w = catmip.dbeta_grid(llk, 0.25)
    assert b == 1.0 and math.isclose(db, 0.75) and cov < 1.0
    assert math.isclose(w.sum(), 1.0, rel_tol=1e-12)


def test_cov_grid_hits_target():
    rng = np.random.default_rng(0)
    llk = rng.normal(-5e4, 2e3, 4096)
    b, db, cov, w = catmip.dbeta_grid(llk, 0.0)
    assert 0 < db < 1 and b == db
    # the grid stops within tolerance of the target or at its resolution
    c_lo, _ = catmip.cov_of(db * (1 - 1e-9), llk, catmip.median_gsl(llk))
    assert abs(cov - 1.0) < 0.01 or cov >= 1.0
    assert np.all(w >= 0) and math.isclose(w.sum(), 1.0, rel_tol=1e-12)


def test_cov_brent_skip_and_target():
    """Brent solver (COV.cc:58-219): skip to β = 1 like the grid, otherwise a δβ whose COV is
    within tolerance of the target, close to the grid's answer, inside [0, 1 - β]."""
    llk = np.linspace(-1.0, -0.999, 1000)
    b, db, cov, w = catmip.dbeta_brent(llk, 0.25)
    assert b == 1.0 and math.isclose(db, 0.75) and cov < 1.0
    rng = np.random.default_rng(0)
    for llk, beta in [(rng.normal(-5e4, 2e3, 4096), 0.0), (-np.exp(rng.uniform(0, 12, 3000)), 0.3)]:
        b, db, cov, w = catmip.dbeta_brent(llk, beta)
        assert 0 < db < 1 - beta and math.isclose(b, beta + db)
        assert abs(cov - 1.0) < 0.01
        _, dbg, covg, _ = catmip.dbeta_grid(llk, beta)
        assert abs(db - dbg) < 0.25 * dbg      # both meet the tolerance; the COV is flat near it
        assert np.all(w >= 0) and math.isclose(w.sum(), 1.0, rel_tol=1e-12)


def test_cov_overflow_sentinel():
    llk = np.array([0.0, 0.0, 1e6, -1e6])
    c, _ = catmip.cov_of(1.0, llk, catmip.median_gsl(llk))
    assert c == 1e100


def test_multiplicities_gsl_semantics():
    w = np.array([0.25, 0.0, 0.5, 0.25])
    r = np.array([0.0, 0.2499, 0.25, 0.74, 0.75, 0.999, 1.0])
    c = catmip.multiplicities(w, r)
    # bins [0,.25) [.25,.25) [.25,.75) [.75,1.0); 1.0 falls beyond the last edge and is dropped
    assert c.tolist() == [2, 0, 2, 2]


def test_rank_order_ties_by_index():
    c = np.array([1, 2, 0, 2, 1])
    assert catmip.rank_order(c).tolist() == [1, 1, 3, 3, 0, 4]
    assert catmip.rank_order(np.array([2, 0, 1, 0])).tolist() == [0, 0, 2, 0]


def test_weighted_cov_matches_numpy():
    rng = np.random.default_rng(1)
    th = rng.normal(size=(500, 3))
    w = rng.random(500)
    w /= w.sum()
    ref = np.cov(th.T, aweights=w, bias=True)
    np.testing.assert_allclose(catmip.weighted_cov(th, w), ref, rtol=1e-10, atol=1e-12)


def test_adapt_scaling_bounds():
    assert catmip.adapt_scaling(0, 10, 0) == 0.1 + 0.0 or math.isclose(catmip.adapt_scaling(0, 10, 0), 1 / 9)
    assert catmip.adapt_scaling(10, 0, 0) == 1.0
    assert math.isclose(catmip.adapt_scaling(5, 5, 0), (8 * 0.5 + 1) / 9)


def test_annealing_gaussian_posterior():
    """1-D linear-Gaussian toy: posterior mean/sd against the analytic answer."""
    rng = np.random.default_rng(5)
    g = rng.normal(size=40)
    truth, sigma = 0.3, 0.5
    d = g * truth + rng.normal(0, sigma, 40)

    def llk(theta):
        r = theta[:, :1] * g[None, :] - d[None, :]
        return -0.5 * np.sum(r * r, 1) / sigma ** 2, np.zeros(theta.shape[0], bool)

    res = catmip.Annealing(llk, [-5.0], [5.0], chains=4000, steps=5, seed=11).run()
    assert res["beta"] == 1.0
    post_var = sigma ** 2 / np.sum(g * g)
    post_mean = np.sum(g * d) / np.sum(g * g)
    th = res["theta"][:, 0]
    assert abs(th.mean() - post_mean) < 4 * math.sqrt(post_var / 4000) * 3
    assert abs(th.std() - math.sqrt(post_var)) < 0.1 * math.sqrt(post_var)
