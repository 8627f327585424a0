"""Linear Gaussian model on the tcgen05 tensor cores against the FP64 oracle.

Tolerance: |llk_tc - llk_ref| <= 1e-5 |llk_ref| + 0.05 for samples spread like a
posterior around the truth, and <= 1e-4 |llk_ref| for samples from the prior (larger
misfits, still the split-BF16 product carries only θ - θ̄); the FP64 path to 1e-10.
"""
import math

import numpy as np
import pytest
import torch

from altar_gb300.distributions import Uniform
from altar_gb300.models import Contiguous, Linear

pytestmark = pytest.mark.gpu


class _App:
    class job:
        chains = 1024

    rng = None
    controller = None


def exp_cov(rng, m, span=50e3, sill=1e-4, corr=2e3):
    xy = rng.uniform(0, span, (m, 2))
    dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
    return sill * np.exp(-dist / corr)


def problem(m, p, seed=0):
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(m, p))
    truth = rng.uniform(-1, 1, p)
    Cd = exp_cov(rng, m)
    L = np.linalg.cholesky(Cd)
    d = G @ truth + L @ rng.normal(size=m)
    return G, d, Cd, truth


def oracle_llk(G, d, Cd, theta):
    r = theta @ G.T - d
    sol = np.linalg.solve(Cd, r.T)
    sign, logdet = np.linalg.slogdet(Cd)
    return -0.5 * (d.size * math.log(2 * math.pi) + logdet) - 0.5 * np.einsum("ij,ji->i", r, sol)


# the last case has 1,024 tiles of 128 chains x 256 observations: each persistent CTA takes
# several tiles and reuses both TMEM accumulators
# (4096, 256, 16384) is the linear-Gaussian workload's size
@pytest.mark.parametrize("m,p,n", [(512, 64, 384), (1024, 256, 1024), (777, 100, 300), (2048, 64, 16384),
                                   (4096, 256, 16384)])
def test_linear_llk_tensor_cores(cuda, m, p, n):
    G, d, Cd, truth = problem(m, p)
    rng = np.random.default_rng(1)
    model = Linear({"theta": Contiguous(p, Uniform((-1, 1)))}, green=G, data=d, cd=Cd)
    app = _App()
    app.job.chains = n
    model.initialize(app)
    post = np.clip(truth[None, :] + 1e-3 * rng.normal(size=(n, p)), -1, 1)
    prior = rng.uniform(-1, 1, (n, p))
    for theta, rel, absn in ((post, 1e-5, 0.05), (prior, 1e-4, 0.0)):
        th = torch.from_numpy(theta).cuda()
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        model.forward(th, out)
        torch.cuda.synchronize()
        assert int(model.flags.item()) == 0
        ref = oracle_llk(G, d, Cd, theta)
        err = np.abs(out.cpu().numpy() - ref)
        assert np.all(err <= rel * np.abs(ref) + absn), (err.max(), np.abs(ref).max())
        model.tensor_cores = False
        model.forward(th, out)
        model.tensor_cores = True
        torch.cuda.synchronize()
        assert np.max(np.abs(out.cpu().numpy() - ref) / np.abs(ref)) < 1e-10


def test_dense_cd_two_source_mogi(cuda):
    """Two Mogi sources, three datasets of uneven size with dense exponential Cd."""
    from altar_gb300.models import DenseMogi
    from oracle import catmip
    rng = np.random.default_rng(3)
    sizes, loss = (300, 520, 190), ([0.38, -0.08, 0.92], [-0.6, 0.1, 0.79], [0.1, 0.55, 0.83])
    truth = np.array([-4e3, 1e3, 3e3, 6.3, 3e3, -2e3, 4e3, 6.1])
    datasets = []
    for m, l in zip(sizes, loss):
        xy = rng.uniform(-25e3, 25e3, (m, 2))
        dist = np.sqrt(((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1))
        cd = 1.6e-5 * np.exp(-dist / 2e3) + 1e-9 * np.eye(m)
        u = catmip.mogi_los(truth[None, :], xy[:, 0], xy[:, 1], np.tile(l, (m, 1)), 0.25, log_strength=True,
                            nsources=2, stride=4)[0]
        d = u + np.linalg.cholesky(cd) @ rng.normal(size=m)
        datasets.append(dict(x=xy[:, 0], y=xy[:, 1], los=l, d=d, cd=cd))
    psets = {}
    for sidx in range(2):
        psets[f"location{sidx}"] = Contiguous(2, Uniform((-1e4, 1e4)))
        psets[f"depth{sidx}"] = Contiguous(1, Uniform((1e3, 8e3)))
        psets[f"source{sidx}"] = Contiguous(1, Uniform((5.0, 7.0)))
    model = DenseMogi(psets, datasets)
    n = 384
    app = _App()
    app.job.chains = n
    model.initialize(app)
    theta = truth[None, :] + rng.normal(size=(n, 8)) * [200, 200, 100, 0.02, 200, 200, 100, 0.02]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    model.forward(torch.from_numpy(theta).cuda(), out)
    torch.cuda.synchronize()
    assert int(model.flags.item()) == 0
    ref = np.zeros(n)
    for ds, m in zip(datasets, sizes):
        u = catmip.mogi_los(theta, ds["x"], ds["y"], np.tile(ds["los"], (m, 1)), 0.25, log_strength=True,
                            nsources=2, stride=4)
        r = u - ds["d"][None, :]
        sign, logdet = np.linalg.slogdet(ds["cd"])
        ref += -0.5 * (m * math.log(2 * math.pi) + logdet) - 0.5 * np.einsum("ij,ji->i", r, np.linalg.solve(ds["cd"], r.T))
    err = np.abs(out.cpu().numpy() - ref)
    assert np.all(err <= 1e-4 * np.abs(ref) + 0.5), (err.max(), np.abs(ref).min())


def test_dense_cd_workload_size(cuda):
    """The batched two-source Mogi workload at its stated size: three datasets of 12,000 /
    30,000 / 7,500 stations with dense exponential Cd and 65,536 chains, evaluated in one
    forward launch plus the tcgen05 whitening of each block; 256 evenly spaced chains are
    checked against the FP64 oracle (numpy Mogi, FP64 Cholesky solves) within 1e-4 relative."""
    from altar_gb300.models import DenseMogi
    from oracle import catmip
    rng = np.random.default_rng(5)
    sizes, loss = (12000, 30000, 7500), ([0.38, -0.08, 0.92], [-0.61, 0.11, 0.78], [0.09, 0.56, 0.82])
    truth = np.array([-4e3, 1e3, 3e3, 6.3, 3e3, -2e3, 4e3, 6.1])
    datasets = []
    for m, l in zip(sizes, loss):
        xy = torch.from_numpy(rng.uniform(-25e3, 25e3, (m, 2))).cuda()
        cd = 1.6e-5 * torch.exp(-torch.cdist(xy, xy) / 2e3) + 1e-9 * torch.eye(m, dtype=torch.float64, device="cuda")
        xy = xy.cpu().numpy()
        u = catmip.mogi_los(truth[None, :], xy[:, 0], xy[:, 1], np.tile(l, (m, 1)), 0.25, log_strength=True,
                            nsources=2, stride=4)[0]
        noise = (torch.linalg.cholesky(cd) @ torch.from_numpy(rng.normal(size=m)).cuda()).cpu().numpy()
        datasets.append(dict(x=xy[:, 0], y=xy[:, 1], los=l, d=u + noise, cd=cd))
    psets = {}
    for sidx in range(2):
        psets[f"location{sidx}"] = Contiguous(2, Uniform((-1e4, 1e4)))
        psets[f"depth{sidx}"] = Contiguous(1, Uniform((1e3, 8e3)))
        psets[f"source{sidx}"] = Contiguous(1, Uniform((5.0, 7.0)))
    model = DenseMogi(psets, datasets)
    n = 65536
    app = _App()
    app.job.chains = n
    model.initialize(app)
    theta = truth[None, :] + rng.normal(size=(n, 8)) * np.tile([500, 500, 300, 0.05], 2)
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    model.forward(torch.from_numpy(theta).cuda(), out)
    torch.cuda.synchronize()
    assert int(model.flags.item()) == 0
    sub = np.arange(0, n, n // 256)[:256]
    ref = np.zeros(sub.size)
    for ds, m in zip(datasets, sizes):
        u = catmip.mogi_los(theta[sub], ds["x"], ds["y"], np.tile(ds["los"], (m, 1)), 0.25, log_strength=True,
                            nsources=2, stride=4)
        r = torch.from_numpy(u - ds["d"][None, :]).cuda()
        L = torch.linalg.cholesky(ds["cd"])
        z = torch.linalg.solve_triangular(L, r.T, upper=False)
        logdet = 2.0 * torch.log(torch.diagonal(L)).sum()
        ref += (-0.5 * (m * math.log(2 * math.pi) + logdet) - 0.5 * (z * z).sum(0)).cpu().numpy()
    got = out.cpu().numpy()[sub]
    rel = np.abs(got - ref) / np.abs(ref)
    print(f"\ndense-Cd workload size: max rel llk error vs FP64 over {sub.size} chains {rel.max():.2e}")
    assert np.all(rel <= 1e-4), rel.max()
