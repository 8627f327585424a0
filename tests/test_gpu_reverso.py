"""Reverso model on the GPU (ag_reverso_llk, FP64) against the reference's forward model
and the FP64 oracle.

Tolerances: displacements 1e-12 relative to the largest component of the sample
(golden vectors from models/reverso/reverso/libreverso.py); log-likelihoods 1e-12
relative (oracle/reverso.py).  The annealing run is compared with the oracle CATMIP loop
on the same Philox streams (posterior means within 4 Monte Carlo standard errors).
"""
import os

import numpy as np
import pytest
import torch

from altar_gb300 import Application
from altar_gb300.bayesian import Annealer
from altar_gb300.distributions import Uniform
from altar_gb300.models import Contiguous, Reverso
from altar_gb300.simulations import RNG, Job
from oracle import catmip, reverso

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "reverso_golden.npz"))
MATERIAL = dict(zip(("G", "v", "mu", "drho", "g"), (float(x) for x in G["material"])))
PRIORS = [(0.4, 0.8), (2500.0, 3500.0), (3500.0, 4500.0), (1500.0, 2500.0), (1500.0, 2500.0), (1.0, 2.0)]


def _psets():
    return {name: Contiguous(1, Uniform(b)) for name, b in zip(reverso.PARAMS, PRIORS)}


class _App:
    """Just enough of an application for Model.initialize outside a run."""

    def __init__(self, chains=16):
        self.job = Job(chains=chains, steps=1)
        self.rng = RNG(0)
        self.controller = None


def _model(txy, d, var, mode):
    return Reverso(_psets(), txy=txy, d=d, var=var, mode=mode, **MATERIAL).initialize(_App())


def test_reverso_displacements_match_reference(cuda):
    txy = G["txy"]
    phi = np.arctan2(txy[:, 2], txy[:, 1])
    zeros = np.zeros_like(txy)
    theta = torch.from_numpy(G["theta"]).cuda()
    for mode, (ce, cn) in (("fast", (np.cos(phi), np.sin(phi))), ("analytic", (np.sin(phi), np.cos(phi)))):
        m = _model(txy, zeros, np.ones_like(txy), mode)
        u = m.displacements(theta).cpu().numpy()
        for i in range(len(G["theta"])):
            ref = np.stack([G["u_r"][i] * ce, G["u_r"][i] * cn, G["u_z"][i]], 1)
            assert np.max(np.abs(u[i] - ref)) <= 1e-12 * np.max(np.abs(ref)), (mode, i)


def test_reverso_llk_matches_oracle_and_skips_masked_rows(cuda):
    txy, d, var = reverso.synthetic_case(**MATERIAL)
    rng = np.random.default_rng(7)
    theta = np.stack([rng.uniform(lo, hi, 512) for lo, hi in PRIORS], 1)
    for mode in ("fast", "analytic"):
        m = _model(txy, d, var, mode)
        out = torch.full((512,), 12345.0, dtype=torch.float64, device="cuda")
        mask = torch.zeros(512, dtype=torch.int32, device="cuda")
        mask[::7] = 1
        m.forward(torch.from_numpy(theta).cuda(), out, mask=mask)
        got = out.cpu().numpy()
        ref = reverso.data_llk(theta, txy, d, var, east_cos=(mode == "fast"), **MATERIAL)
        live = mask.cpu().numpy() == 0
        np.testing.assert_allclose(got[live], ref[live], rtol=1e-12)
        assert np.all(got[~live] == 12345.0)


def test_reverso_annealing_matches_oracle(cuda):
    """The reference's synthetic case (analytic strategy, whose E/N convention the
    generator shares) annealed to β = 1 on the device and by the oracle loop."""
    txy, d, var = reverso.synthetic_case(**MATERIAL)
    chains = 1024
    model = Reverso(_psets(), txy=txy, d=d, var=var, mode="analytic", **MATERIAL)
    app = Application(model, job=Job(chains=chains, steps=5), rng=RNG(4), controller=Annealer())
    app.run()
    step = app.controller.worker.step
    assert step.beta == 1.0
    theta = step.theta.cpu().numpy()
    lo, hi = np.array([b[0] for b in PRIORS]), np.array([b[1] for b in PRIORS])

    def llk(th):
        return reverso.data_llk(th, txy, d, var, east_cos=False, **MATERIAL), np.zeros(th.shape[0], bool)

    ref = catmip.Annealing(llk, lo, hi, chains=chains, steps=5, seed=4).run()
    rt = ref["theta"]
    for j in range(6):
        sd = rt[:, j].std()
        mcse = sd / np.sqrt(chains / 8)
        assert abs(theta[:, j].mean() - rt[:, j].mean()) < 4 * mcse, (j, theta[:, j].mean(), rt[:, j].mean(), sd)
        assert abs(theta[:, j].std() - sd) < 0.5 * sd, j
    # the data log-likelihood the device reports for its final population is the oracle's
    np.testing.assert_allclose(step.data.cpu().numpy(),
                               reverso.data_llk(theta, txy, d, var, east_cos=False, **MATERIAL), rtol=1e-12)
