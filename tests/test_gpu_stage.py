"""Stage kernels on the GPU against the FP64 oracle.

Exactness: resampling counts and row order are bit-exact for identical weights
and uniforms; proposals, covariance and the β schedule agree to FP64
round-off (1e-12 relative); the initial prior sample to one ulp.
"""

import numpy as np
import pytest
import torch

from altar_gb300 import _native
from altar_gb300.bayesian.coolingstep import StageState
from altar_gb300.device import ptr, stream_handle, workspace
from oracle import catmip, philox

from gpu_helpers import dev

pytestmark = pytest.mark.gpu


def _sync():
    torch.cuda.synchronize()


def test_prior_sample_and_llk(cuda):
    n, p, seed = 1000, 5, 77
    lo = np.array([-1.0, 0.0, 10.0, -5e3, 1e5])
    hi = np.array([1.0, 2.0, 20.0, 5e3, 1e7])
    th = torch.zeros(n, p, dtype=torch.float64, device="cuda")
    dlo, dhi = dev(lo), dev(hi)
    _native.call("ag_prior_sample", n, p, ptr(dlo), ptr(dhi), seed, 0, None, ptr(th), stream_handle())
    ref = catmip.prior_sample(seed, n, lo, hi, 0)
    # lo (1 - u) + hi u: the device may fuse one product into an FMA, a few ulps of |lo| + |hi|
    tol = 4 * np.finfo(np.float64).eps * (np.abs(lo) + np.abs(hi))
    assert np.all(np.abs(th.cpu().numpy() - ref) <= tol[None, :])
    prior = torch.zeros(n, dtype=torch.float64, device="cuda")
    mask = torch.zeros(n, dtype=torch.int32, device="cuda")
    th[3, 1] = 2.5
    _native.call("ag_prior_llk", ptr(th), n, p, ptr(dlo), ptr(dhi), ptr(mask), ptr(prior), stream_handle())
    _sync()
    m = mask.cpu().numpy()
    assert m[3] == _native.AG_CHAIN_OUT_OF_SUPPORT and m.sum() == 1
    np.testing.assert_allclose(prior.cpu().numpy(), catmip.uniform_log_prior(ref, lo, hi), rtol=1e-15)


def _state(n, p):
    return StageState(n, p)


@pytest.mark.parametrize("p", [4, 33, 256])
def test_propose_and_accept_match_oracle(cuda, p):
    """Up to 32 parameters one thread per chain, above that one warp per chain."""
    n, seed, step = 4096, 123, 3
    rng = np.random.default_rng(0)
    lo, hi = np.full(p, -1.0), np.full(p, 1.0)
    theta = rng.uniform(-0.9, 0.9, (n, p))
    A = rng.normal(size=(p, p))
    L = np.linalg.cholesky(A @ A.T / p + np.eye(p)) * 0.1
    st = _state(n, p)
    st.chol.copy_(dev(L))
    st.epoch.fill_(5)
    st.beta.fill_(0.3)
    th = dev(theta)
    cand = torch.zeros_like(th)
    mask = torch.zeros(n, dtype=torch.int32, device="cuda")
    cprior = torch.zeros(n, dtype=torch.float64, device="cuda")
    dlo, dhi = dev(lo), dev(hi)
    _native.call("ag_propose", st.struct, ptr(th), n, p, ptr(dlo), ptr(dhi), seed, step, ptr(cand),
                 ptr(mask), ptr(cprior), stream_handle())
    _sync()
    z = philox.proposal_normals(seed, n, p, step, 5)
    ref = theta + z @ L.T
    bad = catmip.uniform_verify(ref, lo, hi)
    ref[bad] = theta[bad]
    assert np.array_equal(mask.cpu().numpy() != 0, bad)
    np.testing.assert_allclose(cand.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)
    # accept
    cdata = dev(rng.normal(-10, 3, n))
    prior = dev(np.full(n, -p * np.log(2.0)))
    data = dev(rng.normal(-10, 3, n))
    post = prior + 0.3 * data
    post_ref = post.cpu().numpy().copy()
    _native.call("ag_accept", st.struct, n, p, seed, step, ptr(mask), ptr(cand), ptr(cprior), ptr(cdata),
                 ptr(th), ptr(prior), ptr(data), ptr(post), stream_handle())
    _sync()
    cpost = cprior.cpu().numpy() + 0.3 * cdata.cpu().numpy()
    u = philox.accept_uniforms(seed, n, step, 5)
    unl = ~bad & (np.log(u) > cpost - post_ref)
    ok = ~bad & ~unl
    cnt = st.counters.cpu().numpy()
    assert cnt.tolist() == [int(ok.sum()), int(bad.sum()), int(unl.sum())]
    got = th.cpu().numpy()
    np.testing.assert_array_equal(got[ok], cand.cpu().numpy()[ok])
    np.testing.assert_array_equal(got[~ok], theta[~ok])


@pytest.mark.parametrize("kind", ["normal", "skip", "overflow", "wide"])
def test_cov_schedule_matches_oracle(cuda, kind):
    rng = np.random.default_rng(4)
    n = 5000
    beta0 = 0.0
    if kind == "normal":
        llk = rng.normal(-3e4, 1e3, n)
    elif kind == "skip":
        llk = rng.normal(-100.0, 1e-4, n)
        beta0 = 0.4
    elif kind == "overflow":
        llk = np.concatenate([rng.normal(-1e6, 1e5, n - 10), rng.normal(0.0, 1.0, 10)])
    else:
        llk = -np.exp(rng.uniform(0, 14, n))
    st = _state(n, 2)
    st.beta.fill_(beta0)
    ws = workspace(_native.load().ag_cov_workspace_bytes(n))
    dllk = dev(llk)
    _native.call("ag_cov_schedule", st.struct, ptr(dllk), n, 1.0, 0.01, ptr(ws), ws.numel(), stream_handle())
    _sync()
    b_ref, db_ref, cov_ref, w_ref = catmip.dbeta_grid(llk, beta0, 1.0, 0.01)
    b, db, cov = st.scalars.cpu().numpy()[:3]
    assert abs(b - b_ref) <= 1e-12 * max(1.0, abs(b_ref)), (b, b_ref)
    assert abs(db - db_ref) <= 1e-12 * max(1e-300, abs(db_ref)) or db == db_ref
    assert abs(cov - cov_ref) <= 1e-9 * max(1.0, cov_ref)
    np.testing.assert_allclose(st.w.cpu().numpy(), w_ref, rtol=1e-10, atol=1e-300)


@pytest.mark.parametrize("kind", ["normal", "skip", "overflow", "wide"])
def test_cov_schedule_brent_matches_oracle(cuda, kind):
    """Brent δβ solver: same decisions as the oracle's restatement.  The device evaluates the
    COV from shifted weight moments and the oracle from the normalised weights, so the
    iterates may differ in the last bits: δβ within 1e-8 relative, COV within 1e-6."""
    rng = np.random.default_rng(5)
    n = 5000
    beta0 = 0.0
    if kind == "normal":
        llk = rng.normal(-3e4, 1e3, n)
    elif kind == "skip":
        llk = rng.normal(-100.0, 1e-4, n)
        beta0 = 0.4
    elif kind == "overflow":
        llk = np.concatenate([rng.normal(-1e6, 1e5, n - 10), rng.normal(0.0, 1.0, 10)])
    else:
        llk = -np.exp(rng.uniform(0, 14, n))
    st = _state(n, 2)
    st.beta.fill_(beta0)
    ws = workspace(_native.load().ag_cov_workspace_bytes(n))
    dllk = dev(llk)
    _native.call("ag_cov_schedule_brent", st.struct, ptr(dllk), n, 1.0, 0.01, 1000, ptr(ws), ws.numel(),
                 stream_handle())
    _sync()
    b_ref, db_ref, cov_ref, w_ref = catmip.dbeta_brent(llk, beta0, 1.0, 0.01, 1000)
    b, db, cov = st.scalars.cpu().numpy()[:3]
    assert abs(db - db_ref) <= 1e-8 * abs(db_ref), (db, db_ref)
    assert abs(b - b_ref) <= 1e-8 * max(abs(b_ref), 1e-300) + 1e-15, (b, b_ref)
    assert abs(cov - cov_ref) <= 1e-6 * max(1.0, cov_ref), (cov, cov_ref)
    if kind != "skip":
        assert abs(cov - 1.0) < 0.01 or cov < 1.0
    np.testing.assert_allclose(st.w.cpu().numpy(), w_ref, rtol=1e-6, atol=1e-300)


@pytest.mark.parametrize("p", [6, 100, 512])
def test_weighted_cov_and_cholesky(cuda, p):
    rng = np.random.default_rng(6)
    n = 3000
    scales = np.resize([1, 2, 3, 1e3, 1e-2, 5], p)
    offsets = np.resize([0, 1, 2, 5e3, 0, -3], p)
    theta = rng.normal(size=(n, p)) * scales + offsets
    w = rng.random(n)
    w /= w.sum()
    st = _state(n, p)
    st.w.copy_(dev(w))
    st.scaling.fill_(0.37)
    ws = workspace(_native.load().ag_sigma_workspace_bytes(n, p))
    dth = dev(theta)
    _native.call("ag_weighted_cov", st.struct, ptr(dth), n, p, ptr(ws), ws.numel(), stream_handle())
    _native.call("ag_cholesky_scaled", st.struct, p, stream_handle())
    _sync()
    ref = catmip.weighted_cov(theta, w)
    np.testing.assert_allclose(st.sigma.cpu().numpy(), ref, rtol=1e-11, atol=1e-11 * np.abs(ref).max())
    L = st.chol.cpu().numpy()
    # entrywise against LAPACK (a different summation order; the columns' scales span 1e-2 to 1e3,
    # so the condition number grows with p), and the backward error of the factorisation
    np.testing.assert_allclose(L, catmip.cholesky_scaled(ref, 0.37), rtol=1e-10 if p <= 32 else 1e-8,
                               atol=1e-12)
    s2 = 0.37 ** 2 * st.sigma.cpu().numpy()
    assert np.abs(L @ L.T - s2).max() <= 1e-13 * np.abs(s2).max()
    assert int(st.flags.item()) == 0
    # not positive definite: flagged, diagonal fallback
    st.sigma.copy_(dev(-np.eye(p)))
    _native.call("ag_cholesky_scaled", st.struct, p, stream_handle())
    _sync()
    assert int(st.flags.item()) & _native.AG_DEV_ERR_NOT_SPD


@pytest.mark.parametrize("n", [1, 2, 777, 32768])
def test_resample_bit_exact(cuda, n):
    rng = np.random.default_rng(n)
    p, seed, epoch = 3, 99, 7
    w = rng.gamma(0.3, size=n)
    w[rng.random(n) < 0.2] = 0.0
    if w.sum() == 0:
        w[0] = 1.0
    w /= w.sum()
    theta = rng.normal(size=(n, p))
    prior, data = rng.normal(size=n), rng.normal(size=n)
    st = _state(n, p)
    st.w.copy_(dev(w))
    st.epoch.fill_(epoch)
    st.beta.fill_(0.25)
    outs = [torch.zeros(n, p, dtype=torch.float64, device="cuda")] + [
        torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    ws = workspace(_native.load().ag_resample_workspace_bytes(n))
    ins = [dev(theta), dev(prior), dev(data)]
    _native.call("ag_resample", st.struct, n, p, seed, *(ptr(t) for t in ins),
                 *(ptr(t) for t in outs), ptr(counts), ptr(ws), ws.numel(), stream_handle())
    _sync()
    c_ref = catmip.multiplicities(w, philox.resample_uniforms(seed, n, epoch))
    assert np.array_equal(counts.cpu().numpy(), c_ref)
    src = catmip.rank_order(c_ref)
    assert np.array_equal(outs[0].cpu().numpy(), theta[src])
    assert np.array_equal(outs[1].cpu().numpy(), prior[src])
    assert np.array_equal(outs[2].cpu().numpy(), data[src])
    np.testing.assert_allclose(outs[3].cpu().numpy(), prior[src] + 0.25 * data[src], rtol=1e-15)


def test_adapt_scaling(cuda):
    st = _state(4, 2)
    st.counters.copy_(torch.tensor([30, 50, 20], dtype=torch.int64, device="cuda"))
    _native.call("ag_adapt_scaling", st.struct, 8.0, 1.0, stream_handle())
    _sync()
    assert abs(st.scaling.item() - catmip.adapt_scaling(30, 50, 20)) < 1e-15
    assert st.counters.cpu().tolist() == [0, 0, 0] and int(st.epoch.item()) == 1
