"""Posterior parity with the oracle CATMIP loop within 2 Monte Carlo standard errors.

The reference (tests/golden/posterior_golden.npz, written by
tests/golden/make_posterior_golden.py) holds, for seeds 1..K, the summaries of the
final population of the FP64 oracle loop (oracle/catmip.py, the reference's
Annealer/COV/Metropolis restated, drawing from the device's Philox streams):
mean and standard deviation of each parameter (Mogi) or of the mode-independent
CDM quantities (centroid, depth, opening, sorted semi-axes).

MCSE.  The spread of a summary over the K oracle seeds is the Monte Carlo standard
error of one run: it is what one run's estimate actually varies by, resampling
correlation included, with no effective-sample-size assumption.  The device runs the
same K seeds on the same inputs.  For each summary q the centre of the K device runs
must lie within 2 standard errors of the centre of the K oracle runs.

Centre and spread are the median over seeds and 1.4826 × the median absolute deviation
(the standard deviation for normal data), and the standard error of the difference of
two medians is sqrt(π/2) · spread · sqrt(2 / K).  Medians, because a CATMIP run
occasionally settles in a secondary mode of the CDM likelihood and ends there: on this
case (2,048 chains, 5 steps per stage) 6 of 60 device seeds ended with their best
log-likelihood ~500 below the others'.  Such a run shifts the mean over 24 seeds by
several standard errors whichever side it falls on, so the mean would measure that
lottery; the median measures the typical run, and a bias of the sampler moves it as it
moves the mean.  The runs more than 5 spreads from the oracle's centre are counted on
both sides and printed.  (Runs with the same seed share their random streams but not
their trajectories: rounding differences in the likelihood change accept decisions.)
"""
import os

import numpy as np
import pytest

from altar_gb300 import Application
from altar_gb300.bayesian import Annealer
from altar_gb300.distributions import Uniform
from altar_gb300.models import CDM, Contiguous, Mogi
from altar_gb300.models.observations import Observations
from altar_gb300.simulations import RNG, Job

pytestmark = pytest.mark.gpu

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "posterior_golden.npz"))
LOS = np.array([0.38, -0.08, 0.92])


def _compare(name, labels, gpu, ref):
    K = ref.shape[0]
    centre_ref, centre_gpu = np.median(ref, 0), np.median(gpu, 0)
    spread = 1.4826 * np.median(np.abs(ref - centre_ref), 0)
    se = np.sqrt(np.pi / 2.0) * spread * np.sqrt(2.0 / K)
    z = (centre_gpu - centre_ref) / se
    out_ref = (np.abs(ref - centre_ref) > 5 * spread).any(1)
    out_gpu = (np.abs(gpu - centre_ref) > 5 * spread).any(1)
    print(f"\n{name}: K = {K} seeds per side; difference of the seed medians in standard errors:")
    for lab, zz, m, g, r in zip(labels, z, spread, centre_gpu, centre_ref):
        print(f"  {lab:>14s}  device {g: .6e}  oracle {r: .6e}  MCSE {m:.3e}  z {zz:+.2f}")
    print(f"  runs more than 5 MCSE from the oracle's centre in some summary: device {out_gpu.sum()} "
          f"(seeds {list(np.nonzero(out_gpu)[0] + 1)}), oracle {out_ref.sum()} (seeds {list(np.nonzero(out_ref)[0] + 1)})")
    return z


def test_mogi_posterior_within_2_mcse(cuda):
    X, Y, d = G["mogi_X"], G["mogi_Y"], G["mogi_d"]
    ref = G["mogi_summaries"]
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
             "source": Contiguous(1, Uniform((1e5, 1e7)))}
    rows, stages = [], []
    for seed in range(1, ref.shape[0] + 1):
        model = Mogi(psets, observations=Observations(X, Y, np.tile(LOS, (X.size, 1)), d, 2.5e-5),
                     log_strength=False)
        app = Application(model, job=Job(chains=1024, steps=5), rng=RNG(seed), controller=Annealer())
        app.run()
        th = app.controller.worker.step.theta.cpu().numpy()
        assert app.controller.worker.step.beta == 1.0
        rows.append(np.concatenate([th.mean(0), th.std(0)]))
        stages.append(len(app.controller.worker.reports))
    labels = [f"mean {p}" for p in ("x", "y", "depth", "dV")] + [f"sd {p}" for p in ("x", "y", "depth", "dV")]
    z = _compare("Mogi workload", labels, np.array(rows), ref)
    print(f"  stages: device {np.mean(stages):.1f}, oracle {G['mogi_stages'].mean():.1f}")
    assert np.all(np.abs(z) <= 2.0), z


def test_cdm_posterior_within_2_mcse(cuda):
    X, Y, d = G["cdm_X"], G["cdm_Y"], G["cdm_d"]
    ref = G["cdm_summaries"]
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 1e4))),
             "opening": Contiguous(1, Uniform((-50, 50))), "a": Contiguous(3, Uniform((100, 3000))),
             "omega": Contiguous(3, Uniform((-90, 90)))}
    rows, stages = [], []
    for seed in range(1, ref.shape[0] + 1):
        model = CDM(psets, observations=Observations(X, Y, np.tile(LOS, (X.size, 1)), d, 9e-6))
        app = Application(model, job=Job(chains=2048, steps=5), rng=RNG(seed), controller=Annealer())
        app.run()
        th = app.controller.worker.step.theta.cpu().numpy()
        assert app.controller.worker.step.beta == 1.0
        q = np.concatenate([th[:, 0:4], np.sort(th[:, 4:7], axis=1)], axis=1)
        rows.append(np.concatenate([q.mean(0), q.std(0)]))
        stages.append(len(app.controller.worker.reports))
    names = ("x", "y", "depth", "opening", "a_min", "a_mid", "a_max")
    labels = [f"mean {p}" for p in names] + [f"sd {p}" for p in names]
    z = _compare("CDM, 576 stations, 2,048 chains", labels, np.array(rows), ref)
    dev_rows = np.array(rows)
    print("  per seed (device - oracle), in MCSE:")
    spread = 1.4826 * np.median(np.abs(ref - np.median(ref, 0)), 0)
    for j, lab in enumerate(labels):
        print(f"  {lab:>14s} " + " ".join("%+.1f" % v for v in (dev_rows[:, j] - ref[:, j]) / spread[j]))
    print(f"  stages: device {np.mean(stages):.1f}, oracle {G['cdm_stages'].mean():.1f}")
    assert np.all(np.abs(z) <= 2.0), z
