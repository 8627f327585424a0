"""FP64 restatement of the CATMIP loop and the Mogi / Gaussian pieces it drives.

Oracle only (test infrastructure).  Each function cites the reference lines
it restates.  Where the reference relies on GSL (RNG streams, histogram
binning order, heap-sort tie order, Brent iterates) parity is unpinned: the
random draws come from ``oracle.philox`` (the device's own streams) and ties
in the resampling order are broken by increasing index, as on the device.
"""
import math

import numpy as np

from . import philox


# --------------------------------------------------------------------------- forward models
def mogi_los(theta, x, y, los, nu, x_idx=0, depth_idx=2, strength_idx=3, log_strength=True,
             nsources=1, stride=0):
    """LOS displacement of Mogi point sources, (N, M) (models/mogi/lib/libmogi/Source.cc:65-118)."""
    theta = np.atleast_2d(np.asarray(theta, dtype=np.float64))
    u = np.zeros((theta.shape[0], np.size(x)))
    for s in range(nsources):
        o = s * stride
        xs = theta[:, x_idx + o, None]
        ys = theta[:, x_idx + 1 + o, None]
        d = theta[:, depth_idx + o, None]
        sv = theta[:, strength_idx + o, None]
        dv = 10.0 ** sv if log_strength else sv
        dx = xs - np.asarray(x)[None, :]
        dy = ys - np.asarray(y)[None, :]
        R = np.sqrt(dx * dx + dy * dy + d * d)
        C = (nu - 1.0) * dv / math.pi
        u += (dx * los[None, :, 0] + dy * los[None, :, 1] - d * los[None, :, 2]) * C / R ** 3
    return u


def diag_llk(pred, d, variance, offsets=None, oid=None):
    """norm - 1/2 Σ r²/σ² with r = pred - d - offset (Native.py:176-186, L2.py:39-52, diagonal Cd)."""
    r = np.asarray(pred) - np.asarray(d)[None, :]
    if offsets is not None:
        r = r - offsets[:, oid]
    var = np.broadcast_to(np.asarray(variance, dtype=np.float64), r.shape[1:])
    norm = -0.5 * (var.size * math.log(2.0 * math.pi) + float(np.sum(np.log(var))))
    return norm - 0.5 * np.sum(r * r / var[None, :], axis=1), r


def llk_from_residuals(resid, weight, norm):
    """FP64 log-likelihood of given residuals: norm - 1/2 Σ w r² (exactly summed)."""
    r = np.asarray(resid, dtype=np.float64)
    w = np.asarray(weight, dtype=np.float64)
    return norm - 0.5 * np.sum(r * r * w[None, :], axis=1)


# --------------------------------------------------------------------------- prior
def uniform_verify(theta, lo, hi):
    """Out-of-support mask (altar/altar/distributions/Uniform.py:45-72, closed interval)."""
    return np.any((theta < lo[None, :]) | (theta > hi[None, :]), axis=1)


def uniform_log_prior(theta, lo, hi):
    """Σ_j log(1/(hi_j - lo_j)) (altar/altar/distributions/Base.py:61-79)."""
    return np.full(theta.shape[0], -float(np.sum(np.log(hi - lo))))


def prior_sample(seed, n, lo, hi, attempt=0):
    """gsl_ran_flat draws a(1-u) + b u on the PRIOR stream."""
    u = philox.prior_uniforms(seed, n, lo.size, attempt)
    return lo[None, :] * (1.0 - u) + hi[None, :] * u


# --------------------------------------------------------------------------- COV schedule
def cov_of(dbeta, llk, median):
    """COV of the normalised weights (altar/lib/libaltar/bayesian/COV.cc:335-368)."""
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        w = np.exp(dbeta * (llk - median))
        wsum = w.size * np.mean(w)
        w = w / wsum
        mean = np.mean(w)
        sd = np.sqrt(np.sum((w - mean) ** 2) / (w.size - 1))
        cov = sd / mean
    if not np.isfinite(cov):
        return 1e100, w
    return float(cov), w


def median_gsl(llk):
    """gsl_stats_median_from_sorted_data of the sorted vector (Grid.py:57)."""
    s = np.sort(llk)
    n = s.size
    return s[(n - 1) // 2] if n % 2 else (s[(n - 1) // 2] + s[n // 2]) / 2.0


def dbeta_grid(llk, beta, target=1.0, tol=0.01):
    """Iterative grid δβ search (COV.cc:222-326). Returns (new β, δβ, cov, w)."""
    median = median_gsl(llk)
    low, high = 0.0, 1.0 - beta
    cov, w = cov_of(high, llk, median)
    if cov < target or abs(cov - target) < tol:
        return 1.0, high, cov, w
    nb_max = 10
    nloop = 0
    found = False
    guess = 0.0
    while True:
        nloop += 1
        step = (high - low) / nb_max
        guess = low
        nb = 0
        while nb <= nb_max:
            c, _ = cov_of(guess, llk, median)
            if abs(c - target) < tol:
                found = True
                break
            if c >= target:
                if nb == 0:
                    found = True
                break
            guess += step
            nb += 1
        if nb > nb_max:
            guess -= step
        high = guess
        low = guess - step
        if not (nloop <= nb_max and not found):
            break
    cov, w = cov_of(guess, llk, median)
    return beta + guess, guess, cov, w


def dbeta_brent(llk, beta, target=1.0, tol=0.01, maxiter=1000):
    """δβ by Brent's minimiser of (cov - target)² (COV.cc:58-219). Returns (new β, δβ, cov, w).

    Set-up as the reference: bracket [0, 1 - β], skip to β = 1 when the full step meets the
    target (COV.cc:103-116), first point the guess 5e-5 (COV.cc:82), interior point at the
    golden section of the bracket, stop when the cov of the latest point is within tol
    (COV.cc:182) or after maxiter iterations, keep the best point (COV.cc:205).  The iteration
    is Brent's published localmin (1973, ch. 5); the reference runs GSL's version of it, which
    is not part of the reference, so the iterates themselves are not pinned to it.
    """
    median = median_gsl(llk)
    high = 1.0 - beta
    cov, w = cov_of(high, llk, median)
    if cov < target or abs(cov - target) < tol:
        return 1.0, high, cov, w

    def f(x):
        c, _ = cov_of(x, llk, median)
        return (1e100 if c >= 1e100 else (c - target) ** 2), c

    golden = 0.3819660112501051
    a, b = 0.0, high
    x = 5.0e-5 if 5.0e-5 < high else 0.5 * high
    v = w_ = a + golden * (b - a)
    fx, _ = f(x)
    fv, _ = f(v)
    fw = fv
    d = e = 0.0
    it = 0
    while True:
        xm = 0.5 * (a + b)
        tol1 = 1.4901161193847656e-08 * abs(x) + 1e-15
        tol2 = 2.0 * tol1
        if abs(x - xm) <= tol2 - 0.5 * (b - a):
            break
        parabolic = False
        if abs(e) > tol1:
            r = (x - w_) * (fx - fv)
            q = (x - v) * (fx - fw)
            pp = (x - v) * q - (x - w_) * r
            q = 2.0 * (q - r)
            if q > 0.0:
                pp = -pp
            else:
                q = -q
            e_prev, e = e, d
            if abs(pp) < abs(0.5 * q * e_prev) and pp > q * (a - x) and pp < q * (b - x):
                d = pp / q
                u = x + d
                if u - a < tol2 or b - u < tol2:
                    d = tol1 if xm >= x else -tol1
                parabolic = True
        if not parabolic:
            e = (a - x) if x >= xm else (b - x)
            d = golden * e
        u = x + d if abs(d) >= tol1 else x + (tol1 if d >= 0.0 else -tol1)
        fu, cu = f(u)
        if fu <= fx:
            if u < x:
                b = x
            else:
                a = x
            v, fv, w_, fw, x, fx = w_, fw, x, fx, u, fu
        else:
            if u < x:
                a = u
            else:
                b = u
            if fu <= fw or w_ == x:
                v, fv, w_, fw = w_, fw, u, fu
            elif fu <= fv or v == x or v == w_:
                v, fv = u, fu
        it += 1
        if abs(cu - target) < tol or it >= maxiter:
            break
    cov, w = cov_of(x, llk, median)
    return beta + x, x, cov, w


# --------------------------------------------------------------------------- covariance and resampling
def weighted_cov(theta, w):
    """θ̄ = Σwθ/Σw; Σ = Σ w θθᵀ - θ̄θ̄ᵀ (altar/altar/bayesian/COV.py:106-156)."""
    mean = (w[:, None] * theta).sum(0) / w.sum()
    S = (theta * w[:, None]).T @ theta
    return S - np.outer(mean, mean)


def cdf_edges(w):
    """[0, w0, w0+w1, ...] accumulated sequentially (COV.py:242-251)."""
    e = np.empty(w.size + 1)
    e[0] = 0.0
    acc = 0.0
    for i, v in enumerate(w.tolist()):
        acc += v
        e[i + 1] = acc
    return e


def multiplicities(w, r):
    """gsl histogram counts of r over the CDF bins; r >= last edge dropped (COV.py:222-239)."""
    e = cdf_edges(w)
    idx = np.searchsorted(e, r, side="right") - 1
    ok = (r >= e[0]) & (r < e[-1])
    counts = np.zeros(w.size, dtype=np.int64)
    np.add.at(counts, idx[ok], 1)
    return counts


def rank_order(counts):
    """Row sources of the resampled set: decreasing count, ties by increasing index (COV.py:181-206)."""
    order = sorted(range(counts.size), key=lambda i: (-counts[i], i))
    src = [i for i in order for _ in range(int(counts[i]))]
    while len(src) < counts.size:          # dropped uniforms: repeat the first row
        src.append(src[0])
    return np.array(src, dtype=np.int64)


# --------------------------------------------------------------------------- Metropolis
def cholesky_scaled(sigma, scaling):
    return np.linalg.cholesky(scaling * scaling * sigma)


def adapt_scaling(accepted, rejected, unlikely, aw=8.0, rw=1.0):
    """kc = (aw acc + rw)/(aw + rw) in [0.1, 1] (altar/altar/bayesian/Metropolis.py:262-281)."""
    acc = accepted / (accepted + rejected + unlikely)
    return min(1.0, max(0.1, (aw * acc + rw) / (aw + rw)))


class Annealing:
    """The CATMIP loop (altar/altar/bayesian/Annealer.py:79-135) for a data-llk function.

    ``data_llk(theta) -> (llk, invalid_mask)``.  Draws use the device's Philox
    streams, so with identical inputs the oracle and the GPU make the same
    random choices up to floating-point ties.
    """

    def __init__(self, data_llk, lo, hi, chains, steps=5, seed=0, tolerance=1e-3, target=1.0,
                 grid_tol=0.01, scaling=0.1, solver="grid"):
        self.data_llk, self.lo, self.hi = data_llk, np.asarray(lo, float), np.asarray(hi, float)
        self.solver = dbeta_brent if solver == "brent" else dbeta_grid
        self.n, self.p, self.steps, self.seed = chains, self.lo.size, steps, seed
        self.tolerance, self.target, self.grid_tol, self.scaling0 = tolerance, target, grid_tol, scaling

    def initial(self, max_attempts=1000):
        theta = prior_sample(self.seed, self.n, self.lo, self.hi)
        for attempt in range(1, max_attempts + 1):
            llk, bad = self.data_llk(theta)
            if not np.any(bad):
                return theta, llk
            redo = prior_sample(self.seed, self.n, self.lo, self.hi, attempt)
            theta[bad] = redo[bad]
        raise RuntimeError("no valid initial sample")

    def run(self, max_stages=1000, shards=None):
        """shards: an exchange with ``bounds(n) -> (first row, rows)``, ``gather(*arrays)`` and
        ``sum(array)`` (torch tensors sharing the numpy arrays' memory): each rank walks its
        block of rows with the streams of their global indices, then the blocks and the
        accept counters are exchanged and the cool phase runs on the whole population."""
        n, p = self.n, self.p
        theta, data = self.initial()
        prior = uniform_log_prior(theta, self.lo, self.hi)
        beta, scaling, epoch = 0.0, self.scaling0, 0
        post = prior + beta * data
        stages = []
        while beta + self.tolerance < 1 and len(stages) < max_stages:
            beta, dbeta, cov, w = self.solver(data, beta, self.target, self.grid_tol)
            sigma = weighted_cov(theta, w)
            counts = multiplicities(w, philox.resample_uniforms(self.seed, n, epoch))
            src = rank_order(counts)
            theta, prior, data = theta[src].copy(), prior[src].copy(), data[src].copy()
            post = prior + beta * data
            L = cholesky_scaled(sigma, scaling)
            c0, m = (0, n) if shards is None else shards.bounds(n)
            rows = slice(c0, c0 + m)
            th, pr, da, po = theta[rows], prior[rows], data[rows], post[rows]    # views
            acc = rej = unl = 0
            for k in range(self.steps):
                z = philox.proposal_normals(self.seed, n, p, k, epoch)[rows]
                cand = th + z @ L.T
                bad = uniform_verify(cand, self.lo, self.hi)
                cand[bad] = th[bad]
                cprior = uniform_log_prior(cand, self.lo, self.hi)
                cdata, invalid = self.data_llk(cand)
                bad = bad | invalid
                cpost = cprior + beta * cdata
                u = philox.accept_uniforms(self.seed, n, k, epoch)[rows]
                unlikely = ~bad & (np.log(u) > cpost - po)
                ok = ~bad & ~unlikely
                th[ok], pr[ok], da[ok], po[ok] = cand[ok], cprior[ok], cdata[ok], cpost[ok]
                acc += int(ok.sum()); rej += int(bad.sum()); unl += int(unlikely.sum())
            if shards is not None:
                import torch
                shards.gather(*(torch.from_numpy(a) for a in (theta, prior, data, post)))
                c = torch.tensor([acc, rej, unl], dtype=torch.int64)
                shards.sum(c)
                acc, rej, unl = (int(v) for v in c)
            scaling = adapt_scaling(acc, rej, unl)
            epoch += 1
            stages.append(dict(beta=beta, dbeta=dbeta, cov=cov, accepted=acc, rejected=rej,
                               unlikely=unl, scaling=scaling))
        return dict(theta=theta, prior=prior, data=data, posterior=post, beta=beta, stages=stages)
