"""The device side of chain sharding on one GPU: a population walked as two blocks (each with
its global first chain, as two ranks would walk them, here one after the other in one
process) ends where the whole-population walk ends, bit for bit."""
import numpy as np
import pytest
import torch

from altar_gb300 import Application
from altar_gb300.bayesian import Annealer
from altar_gb300.bayesian.sharding import _Block
from altar_gb300.distributions import Uniform
from altar_gb300.models import Contiguous, Mogi
from altar_gb300.models.observations import Observations
from altar_gb300.simulations import RNG, Job
from oracle import catmip

pytestmark = pytest.mark.gpu


def _app(chains):
    g = np.linspace(-15e3, 15e3, 16)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    d = catmip.mogi_los(np.array([[1e3, -2e3, 3e3, 2e6]]), X, Y, los, 0.25, log_strength=False)[0] + \
        np.random.default_rng(7).normal(0, 5e-3, X.size)
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
             "source": Contiguous(1, Uniform((1e5, 1e7)))}
    model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
    return Application(model, job=Job(chains=chains, steps=3), rng=RNG(11), controller=Annealer(graphs=False))


def _copy(step):
    c = step.clone()
    c.state.epoch.copy_(step.state.epoch)
    c.state.chol.copy_(step.state.chol)
    return c


def test_block_walks_equal_the_whole_walk(cuda):
    app = _app(512)
    app.initialize()
    ann = app.controller
    w = ann.worker
    with torch.cuda.stream(w.stream):
        ann.model = app.model
        w.start(annealer=ann)
        w.cool(annealer=ann)                       # β, Σ and the resampled population
        whole, split = _copy(w.step), _copy(w.step)
        ann.sampler.samplePosterior(annealer=ann, step=whole)
        for c0 in (0, 256):
            ann.sampler.samplePosterior(annealer=ann, step=_Block(split, c0, 256))
        torch.cuda.synchronize()
    for name in ("theta", "prior", "data", "posterior"):
        np.testing.assert_array_equal(getattr(split, name).cpu().numpy(), getattr(whole, name).cpu().numpy(),
                                      err_msg=name)
    assert torch.equal(split.state.counters, whole.state.counters)
    assert int(whole.state.counters[0]) > 0
