"""Full CATMIP runs on the GPU through the plugin surface.

The Mogi workload with a single point source, 1,024 LOS points on a 32x32
grid over ±15 km, 1,024 chains and 5 steps per stage is run on the device and
by the FP64 oracle loop with the same Philox streams; posterior means and
standard deviations must agree within a few Monte Carlo standard errors.
"""
import numpy as np
import pytest
import torch

from altar_gb300 import Application
from altar_gb300.bayesian import COV, Annealer, Brent
from altar_gb300.distributions import Uniform
from altar_gb300.models import CDM, Contiguous, Mogi
from altar_gb300.models.observations import Observations
from altar_gb300.simulations import RNG, Checkpoint, Job
from oracle import catmip

from gpu_helpers import cdm_los_oracle, cdm_prior_rows

pytestmark = pytest.mark.gpu

LOS = np.array([0.38, -0.08, 0.92])


def mogi_problem(seed=0):
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    truth = np.array([[0.0, 0.0, 3e3, 2e6]])
    rng = np.random.default_rng(seed)
    d = catmip.mogi_los(truth, X, Y, los, 0.25, log_strength=False)[0] + rng.normal(0, 5e-3, X.size)
    return X, Y, los, d


def mogi_app(chains=1024, steps=5, seed=1, graphs=True, scheduler=None, checkpoint=None, resume=None):
    X, Y, los, d = mogi_problem()
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
             "source": Contiguous(1, Uniform((1e5, 1e7)))}
    model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
    return Application(model, job=Job(chains=chains, steps=steps), rng=RNG(seed),
                       controller=Annealer(graphs=graphs, scheduler=scheduler, checkpoint=checkpoint,
                                           resume=resume))


def test_mogi_posterior_matches_oracle(cuda):
    app = mogi_app()
    app.run()
    step = app.controller.worker.step
    theta = step.theta.cpu().numpy()
    assert step.beta == 1.0
    X, Y, los, d = mogi_problem()
    lo = np.array([-1e4, -1e4, 1e3, 1e5])
    hi = np.array([1e4, 1e4, 8e3, 1e7])

    def llk(th):
        u = catmip.mogi_los(th, X, Y, los, 0.25, log_strength=False)
        return catmip.diag_llk(u, d, np.full(X.size, 2.5e-5))[0], np.zeros(th.shape[0], bool)

    ref = catmip.Annealing(llk, lo, hi, chains=1024, steps=5, seed=1).run()
    rt = ref["theta"]
    nst_gpu, nst_ref = len(app.controller.worker.reports), len(ref["stages"])
    assert abs(nst_gpu - nst_ref) <= max(2, nst_ref // 5), (nst_gpu, nst_ref)
    for j in range(4):
        sd = rt[:, j].std()
        mcse = sd / np.sqrt(1024 / 8)      # resampled chains are strongly correlated
        assert abs(theta[:, j].mean() - rt[:, j].mean()) < 4 * mcse, j
        assert abs(theta[:, j].std() - sd) < 0.5 * sd, j


def test_mogi_posterior_brent_matches_oracle(cuda):
    """The same workload with the Brent δβ solver (Brent.py) on the device and in the oracle."""
    app = mogi_app(scheduler=COV(solver=Brent()))
    app.run()
    step = app.controller.worker.step
    theta = step.theta.cpu().numpy()
    assert step.beta == 1.0
    X, Y, los, d = mogi_problem()
    lo = np.array([-1e4, -1e4, 1e3, 1e5])
    hi = np.array([1e4, 1e4, 8e3, 1e7])

    def llk(th):
        u = catmip.mogi_los(th, X, Y, los, 0.25, log_strength=False)
        return catmip.diag_llk(u, d, np.full(X.size, 2.5e-5))[0], np.zeros(th.shape[0], bool)

    ref = catmip.Annealing(llk, lo, hi, chains=1024, steps=5, seed=1, solver="brent").run()
    rt = ref["theta"]
    reps = app.controller.worker.reports
    assert abs(len(reps) - len(ref["stages"])) <= max(2, len(ref["stages"]) // 5)
    assert all(abs(r["cov"] - 1.0) < 0.01 or r["beta"] == 1.0 for r in reps)
    for j in range(4):
        sd = rt[:, j].std()
        mcse = sd / np.sqrt(1024 / 8)
        assert abs(theta[:, j].mean() - rt[:, j].mean()) < 4 * mcse, j
        assert abs(theta[:, j].std() - sd) < 0.5 * sd, j


def test_checkpoint_resume_repeats_the_run(cuda, tmp_path):
    """8 stages straight and 4 + 4 with a restart from the stage-4 checkpoint give the same
    sample bit for bit (every draw is keyed by seed, epoch and step)."""
    def stages(app, k):
        app.initialize()
        app.controller.posterior(app.model, max_stages=k)
        w = app.controller.worker
        return w.step.theta.cpu().numpy(), w.step.beta, len(w.reports)

    straight, beta_s, _ = stages(mogi_app(seed=3), 8)
    ck = Checkpoint(str(tmp_path / "stage.npz"))
    stages(mogi_app(seed=3, checkpoint=ck), 4)
    resumed, beta_r, n_r = stages(mogi_app(seed=3, resume=ck.path), 4)
    assert n_r == 4 and beta_r == beta_s
    np.testing.assert_array_equal(resumed, straight)


def test_graph_replay_matches_eager(cuda):
    """Captured stage graphs reproduce the eager launches bit for bit."""
    a = mogi_app(chains=512, steps=3, seed=5, graphs=True)
    b = mogi_app(chains=512, steps=3, seed=5, graphs=False)
    a.run()
    b.run()
    ta, tb = a.controller.worker.step.theta.cpu(), b.controller.worker.step.theta.cpu()
    assert torch.equal(ta, tb)
    assert [r["beta"] for r in a.controller.worker.reports] == [r["beta"] for r in b.controller.worker.reports]


def test_cdm_annealing_runs(cuda):
    g = np.linspace(-20e3, 20e3, 24)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    truth = cdm_prior_rows(1, seed=21)
    rng = np.random.default_rng(2)
    d = cdm_los_oracle(truth, X, Y, los)[0] + rng.normal(0, 3e-3, X.size)
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 1e4))),
             "opening": Contiguous(1, Uniform((-50, 50))), "a": Contiguous(3, Uniform((100, 3000))),
             "omega": Contiguous(3, Uniform((-90, 90)))}
    model = CDM(psets, observations=Observations(X, Y, los, d, 9e-6))
    app = Application(model, job=Job(chains=512, steps=3), rng=RNG(3))
    app.initialize()
    rc = app.controller.posterior(model, max_stages=4)
    assert rc == 0
    reps = app.controller.worker.reports
    assert len(reps) == 4 and all(0 < r["beta"] <= 1 for r in reps)
    assert reps[-1]["beta"] > reps[0]["beta"]
    th = app.controller.worker.step.theta.cpu().numpy()
    assert np.all(np.isfinite(th)) and np.all(np.isfinite(app.controller.worker.step.data.cpu().numpy()))


def test_early_rejection_keeps_the_chains(cuda):
    """Early rejection (the CDM evaluation of a candidate stops once its partial
    log-likelihood is below the accept test's floor) changes no accept decision: a CDM run
    with it and one without end with the same θ, log-likelihoods and acceptance counts, bit
    for bit, over the whole run to β = 1 (the work saved is reported)."""
    from altar_gb300.bayesian import Metropolis
    g = np.linspace(-20e3, 20e3, 40)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    truth = cdm_prior_rows(1, seed=21)
    d = cdm_los_oracle(truth, X, Y, los)[0] + np.random.default_rng(2).normal(0, 3e-3, X.size)
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 1e4))),
             "opening": Contiguous(1, Uniform((-50, 50))), "a": Contiguous(3, Uniform((100, 3000))),
             "omega": Contiguous(3, Uniform((-90, 90)))}
    out = {}
    for early in (False, True):
        model = CDM(psets, observations=Observations(X, Y, los, d, 9e-6))
        app = Application(model, job=Job(chains=1024, steps=5), rng=RNG(7),
                          controller=Annealer(sampler=Metropolis(early_reject=early)))
        app.run()
        w = app.controller.worker
        assert w.step.beta == 1.0
        out[early] = ([t.cpu().numpy() for t in (w.step.theta, w.step.prior, w.step.data, w.step.posterior)],
                      [(r["accepted"], r["rejected"], r["unlikely"]) for r in w.reports])
    for a, b in zip(out[False][0], out[True][0]):
        np.testing.assert_array_equal(a, b)
    assert out[False][1] == out[True][1]


def test_forward_floor_semantics(cuda):
    """ag_forward_llk_floor: a chain whose log-likelihood is below its floor may stop with
    -inf; every other chain gets exactly ag_forward_llk's value."""
    from gpu_helpers import cdm_strategy, dev
    g = np.linspace(-20e3, 20e3, 60)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(64, seed=23)
    d = np.random.default_rng(5).normal(0, 3e-3, X.size)
    strat, _ = cdm_strategy(X, Y, los, d, np.full(X.size, 9e-6))
    th = dev(theta)
    full = torch.empty(64, dtype=torch.float64, device="cuda")
    strat.forward(th, full)
    f = full.cpu().numpy()
    floor = np.full(64, -np.inf)
    floor[::4] = f[::4] + 1.0               # certainly below: may stop
    floor[1::4] = f[1::4] - 1.0             # above its floor: must be exact
    floor[2::4] = np.inf                    # stops at the first tile
    got = torch.empty(64, dtype=torch.float64, device="cuda")
    strat.forward(th, got, floor=dev(floor))
    g_ = got.cpu().numpy()
    exact = np.r_[1:64:4, 3:64:4]
    np.testing.assert_array_equal(g_[exact], f[exact])
    assert np.all(np.isneginf(g_[2::4]))
    assert np.all((g_[::4] == f[::4]) | np.isneginf(g_[::4]))


def test_profiler_times_the_phases(cuda, tmp_path):
    """A run with the Profiler registered (phases launched one by one, timed with CUDA
    events) writes the reference's profile file and ends where the captured-graph run ends."""
    import csv

    from altar_gb300.bayesian import Profiler
    app = mogi_app(chains=256, steps=2)
    prof = Profiler(directory=str(tmp_path))
    app.monitors["profiler"] = prof
    app.run()
    assert prof.filename.endswith(f"prof-00000-{prof.beta:03d}x004x000256x002.csv")
    with open(prof.filename, newline="") as f:
        rows = {r[0]: r[1:] for r in csv.reader(f)}
    t = {k: float(v[0]) for k, v in rows.items() if v and k not in ("beta steps", "parameters", "chains", "steps")}
    assert t["simulation"] >= t["beta"] >= t["walk"] >= t["samplePosterior"] > 0
    assert t["data"] > 0 and t["verify"] > 0 and t["accept"] > 0 and t["resample"] > 0
    ref = mogi_app(chains=256, steps=2)
    ref.run()
    np.testing.assert_array_equal(app.controller.worker.step.theta.cpu().numpy(),
                                  ref.controller.worker.step.theta.cpu().numpy())
