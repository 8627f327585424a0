"""Surrogate network and delayed acceptance on the GPU against FP64 oracles.

Tolerances: network outputs and gradients within 1e-4 (normwise, relative) of the FP64
oracle evaluated with the same BF16-rounded weights (the device accumulates in FP32);
Adam within 1e-6; the PCA-space log-likelihood within 1e-9 of the direct sum;
delayed-acceptance decisions identical for identical uniforms.
"""
import ctypes

import numpy as np
import pytest
import torch

from altar_gb300 import Application, _native
from altar_gb300.bayesian import Annealer, DelayedAcceptance, SubsetSurrogate, Surrogate
from altar_gb300.bayesian.coolingstep import StageState
from altar_gb300.device import ptr, stream_handle
from altar_gb300.distributions import Uniform
from altar_gb300.models import Contiguous, Mogi
from altar_gb300.models.observations import Observations
from altar_gb300.simulations import RNG, Job
from oracle import catmip, mlp, philox

from gpu_helpers import LOS, cdm_prior_rows, cdm_strategy, dev

pytestmark = pytest.mark.gpu
SIZES = (10, 256, 256, 256, 256, 64)


def _bf16_round(a):
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()


def _oracle_params(sur):
    flat = sur.params.cpu().numpy().astype(np.float64)
    out, o = [], 0
    for fi, fo in zip(SIZES[:-1], SIZES[1:]):
        W = _bf16_round(flat[o:o + fo * fi].reshape(fo, fi)); o += fo * fi
        b = flat[o:o + fo]; o += fo
        out.append((W, b))
    return out


def _flat(grads):
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def test_mlp_forward_backward_adam(cuda):
    sur = Surrogate(SIZES, seed=3).init_params()
    rng = np.random.default_rng(0)
    n = 512
    x = rng.uniform(-1, 1, (n, 10))
    y = rng.normal(size=(n, 64))
    lib = _native.load()
    net = ctypes.byref(sur.net)
    acts = torch.empty(lib.ag_mlp_activation_floats(net, n), dtype=torch.float32, device="cuda")
    xd, yd = dev(x, torch.float32), dev(y, torch.float32)
    out = torch.empty(n, 64, dtype=torch.float32, device="cuda")
    s = stream_handle()
    _native.call("ag_mlp_forward", net, ptr(sur.params), ptr(sur.pbf), ptr(xd), n, ptr(out), ptr(acts), s)
    P = _oracle_params(sur)
    ref, _ = mlp.forward(P, xd.double().cpu().numpy())
    got = out.double().cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref))
    dout = torch.empty_like(out)
    _native.call("ag_mse_grad", n, 64, ptr(out), ptr(yd), ptr(dout), None, s)
    scratch = torch.empty(2 * n * 256, dtype=torch.float32, device="cuda")
    _native.call("ag_mlp_backward", net, ptr(sur.params), ptr(sur.pbf), ptr(xd), n, ptr(acts), ptr(dout),
                 ptr(sur.grads), ptr(scratch), s)
    g_ref = _flat(mlp.backward(P, xd.double().cpu().numpy(), yd.double().cpu().numpy()))
    g = sur.grads.double().cpu().numpy()
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)
    # one Adam step on the FP32 master copy
    p0 = sur.params.double().cpu().numpy()
    _native.call("ag_adam_step", sur.params.numel(), ptr(sur.params), ptr(sur.grads), ptr(sur.m), ptr(sur.v), 1,
                 1e-3, 0.9, 0.999, 1e-8, ptr(sur.pbf), s)
    torch.cuda.synchronize()
    mh = (0.1 * g) / 0.1
    vh = (0.001 * g * g) / 0.001
    expect = p0 - 1e-3 * mh / (np.sqrt(vh) + 1e-8)
    np.testing.assert_allclose(sur.params.double().cpu().numpy(), expect, rtol=1e-5, atol=1e-7)


def test_training_reduces_loss(cuda):
    sur = Surrogate((10, 64, 64, 8), seed=1, batch=1024).init_params()
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (16384, 10)).astype(np.float32)
    W = rng.normal(size=(10, 8)) / 3
    y = (x @ W + 0.3 * (x @ W) ** 2).astype(np.float32)      # smooth, like a local forward field
    sur.reserve(16384, 10)
    sur.add(dev(x, torch.float32), dev(y, torch.float32))
    losses = sur.train(epochs=10, lr=3e-3)
    assert losses[-1] < 0.1 * losses[0], losses


def test_surrogate_llk_formula(cuda):
    rng = np.random.default_rng(2)
    M, K, n = 700, 16, 64
    B, _ = np.linalg.qr(rng.normal(size=(M, K)))
    mu = rng.normal(size=M)
    d = rng.normal(size=M)
    w = rng.uniform(0.5, 2.0, M)
    scale = rng.uniform(0.5, 3.0, K)
    c = rng.normal(size=(n, K))
    G = B.T @ (w[:, None] * B)
    h = B.T @ (w * (d - mu))
    q0 = float(((mu - d) ** 2 * w).sum())
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    args = [dev(c, torch.float32), dev(scale, torch.float32), dev(G, torch.float32), dev(h, torch.float32)]
    _native.call("ag_surrogate_llk", n, K, *(ptr(a) for a in args), q0, -7.0, ptr(out), stream_handle())
    cf = args[0].double().cpu().numpy() * args[1].double().cpu().numpy()
    u = mu[None, :] + cf @ B.T
    ref = -7.0 - 0.5 * ((u - d) ** 2 * w).sum(1)
    assert np.max(np.abs(out.cpu().numpy() - ref) / np.abs(ref)) < 1e-5


def test_delayed_acceptance_decisions(cuda):
    rng = np.random.default_rng(5)
    n, p, seed, step, epoch = 5000, 3, 17, 2, 4
    st = StageState(n, p)
    st.beta.fill_(0.7)
    st.epoch.fill_(epoch)
    mask = (rng.random(n) < 0.1).astype(np.int32)
    prior = np.full(n, -1.0)
    cprior = np.full(n, -1.0)
    sur, csur = rng.normal(-50, 2, n), rng.normal(-50, 2, n)
    data, cdata = sur + rng.normal(0, 0.5, n), csur + rng.normal(0, 0.5, n)
    post = prior + 0.7 * data
    theta, cand = rng.normal(size=(n, p)), rng.normal(size=(n, p))
    T = {k: dev(v) for k, v in dict(prior=prior, cprior=cprior, sur=sur, csur=csur, data=data, cdata=cdata,
                                   post=post, theta=theta, cand=cand).items()}
    dmask = dev(mask, torch.int32)
    passed = torch.zeros(n, dtype=torch.int32, device="cuda")
    index = torch.zeros(n, dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = stream_handle()
    _native.call("ag_da_screen", st.struct, n, seed, step, ptr(dmask), ptr(T["cprior"]), ptr(T["csur"]),
                 ptr(T["prior"]), ptr(T["sur"]), ptr(passed), ptr(index), ptr(count), s)
    screened = torch.zeros(1, dtype=torch.int64, device="cuda")
    _native.call("ag_da_accept", st.struct, n, p, seed, step, ptr(dmask), ptr(passed), ptr(T["cand"]),
                 ptr(T["cprior"]), ptr(T["cdata"]), ptr(T["csur"]), ptr(T["theta"]), ptr(T["prior"]),
                 ptr(T["data"]), ptr(T["post"]), ptr(T["sur"]), ptr(screened), s)
    torch.cuda.synchronize()
    units = np.arange(n, dtype=np.uint64)
    r1 = philox.draw(seed, units, 1, philox.STREAM_ACCEPT, step, epoch)
    r2 = philox.draw(seed, units, 2, philox.STREAM_ACCEPT, step, epoch)
    u1, u2 = philox.u01_open_closed(r1[0], r1[1]), philox.u01_open_closed(r2[0], r2[1])
    d1 = (cprior + 0.7 * csur) - (prior + 0.7 * sur)
    pass_ref = (mask == 0) & (np.log(u1) <= d1)
    assert np.array_equal(passed.cpu().numpy() != 0, pass_ref)
    assert int(count.item()) == int(pass_ref.sum())
    assert sorted(index.cpu().numpy()[: int(count.item())].tolist()) == np.flatnonzero(pass_ref).tolist()
    cp = cprior + 0.7 * cdata
    acc = pass_ref & (np.log(u2) <= (cp - post) - d1)
    got = T["theta"].cpu().numpy()
    assert np.array_equal(got[acc], cand[acc]) and np.array_equal(got[~acc], theta[~acc])
    cnt = st.counters.cpu().numpy()
    assert cnt.tolist() == [int(acc.sum()), int(mask.sum()), int(n - acc.sum() - mask.sum())]
    assert int(screened.item()) == int(pass_ref.sum())


def test_forward_subset_matches_full(cuda):
    g = np.linspace(-20e3, 20e3, 20)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(40, seed=6)
    strat, _ = cdm_strategy(X, Y, los, np.zeros(X.size), np.full(X.size, 9e-6))
    th = dev(theta)
    full = torch.empty(40, dtype=torch.float64, device="cuda")
    strat.forward(th, full)
    sub = torch.full((40,), -1.0, dtype=torch.float64, device="cuda")
    pick = np.array([3, 7, 8, 21, 39, 0], dtype=np.int32)
    index = torch.zeros(40, dtype=torch.int32, device="cuda")
    index[: pick.size] = dev(pick, torch.int32)
    count = torch.tensor([pick.size], dtype=torch.int32, device="cuda")
    _native.call("ag_forward_llk_subset", strat.kind, ctypes.byref(strat.layout), ptr(th), 40,
                 strat.stations.struct, strat.norm, ptr(index), ptr(count), ptr(sub), None, None, ptr(strat._ws),
                 strat._ws_bytes, stream_handle())
    torch.cuda.synchronize()
    f, sb = full.cpu().numpy(), sub.cpu().numpy()
    assert np.array_equal(sb[pick], f[pick])
    rest = np.setdiff1d(np.arange(40), pick)
    assert np.all(sb[rest] == -1.0)


def test_delayed_acceptance_posterior(cuda):
    """Mogi workload: the DA sampler targets the same posterior as plain Metropolis."""
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    rng = np.random.default_rng(0)
    d = catmip.mogi_los(np.array([[0.0, 0.0, 3e3, 2e6]]), X, Y, los, 0.25, log_strength=False)[0]
    d = d + rng.normal(0, 5e-3, X.size)

    def run(sampler, seed):
        psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
                 "source": Contiguous(1, Uniform((1e5, 1e7)))}
        model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
        app = Application(model, job=Job(chains=2048, steps=5), rng=RNG(seed),
                          controller=Annealer(sampler=sampler))
        app.run()
        return app.controller.worker

    plain = run(None, 7)
    sur = Surrogate((4, 128, 128, 32), seed=2, batch=512, lr=2e-3)
    da = DelayedAcceptance(surrogate=sur, rms_limit=50.0, delta_limit=float("inf"), fit_chains=1024,
                           check_chains=128, epochs=20, inner=1, outer=None, stop_beta=1.0)
    dw = run(da, 7)
    assert sur.trained and any(r.get("mode") == "da" for r in dw.reports)
    tp, td = plain.step.theta.cpu().numpy(), dw.step.theta.cpu().numpy()
    for j in range(4):
        sd = tp[:, j].std()
        assert abs(td[:, j].mean() - tp[:, j].mean()) < 4 * sd / np.sqrt(2048 / 8), j
        assert abs(td[:, j].std() - sd) < 0.5 * sd, j


def test_surrogate_transition_posterior(cuda):
    """k surrogate moves per exact correction still target the exact posterior."""
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    rng = np.random.default_rng(0)
    d = catmip.mogi_los(np.array([[0.0, 0.0, 3e3, 2e6]]), X, Y, los, 0.25, log_strength=False)[0]
    d = d + rng.normal(0, 5e-3, X.size)

    def run(sampler):
        psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
                 "source": Contiguous(1, Uniform((1e5, 1e7)))}
        model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
        app = Application(model, job=Job(chains=2048, steps=5), rng=RNG(9), controller=Annealer(sampler=sampler))
        app.run()
        return app.controller.worker

    plain = run(None)
    sur = Surrogate((4, 128, 128, 32), seed=2, batch=512, lr=2e-3)
    da = DelayedAcceptance(surrogate=sur, rms_limit=50.0, delta_limit=float("inf"), fit_chains=1024,
                           check_chains=128, epochs=20,
                           inner=3, outer=2, stop_beta=1.0)
    dw = run(da)
    assert any(r.get("mode") == "da" for r in dw.reports)
    tp, td = plain.step.theta.cpu().numpy(), dw.step.theta.cpu().numpy()
    for j in range(4):
        sd = tp[:, j].std()
        assert abs(td[:, j].mean() - tp[:, j].mean()) < 4 * sd / np.sqrt(2048 / 8), j
        assert abs(td[:, j].std() - sd) < 0.5 * sd, j


def test_subset_surrogate_transition_posterior(cuda):
    """The coarse (every k-th station) likelihood as the first stage, with the stride picked
    per stage from three levels: the exact correction keeps the posterior of plain Metropolis."""
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    rng = np.random.default_rng(0)
    d = catmip.mogi_los(np.array([[0.0, 0.0, 3e3, 2e6]]), X, Y, los, 0.25, log_strength=False)[0]
    d = d + rng.normal(0, 5e-3, X.size)

    def run(sampler):
        psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
                 "source": Contiguous(1, Uniform((1e5, 1e7)))}
        model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
        app = Application(model, job=Job(chains=2048, steps=5), rng=RNG(9), controller=Annealer(sampler=sampler))
        app.run()
        return app.controller.worker

    plain = run(None)
    sur = SubsetSurrogate(strides=(16, 8, 4))
    da = DelayedAcceptance(surrogate=sur, delta_limit=1.0, check_chains=128, inner=10, outer=1, stop_beta=1.0)
    dw = run(da)
    used = [r.get("stride") for r in dw.reports if r.get("mode") == "da"]
    assert used and set(used) <= {16, 8, 4}
    tp, td = plain.step.theta.cpu().numpy(), dw.step.theta.cpu().numpy()
    for j in range(4):
        sd = tp[:, j].std()
        assert abs(td[:, j].mean() - tp[:, j].mean()) < 4 * sd / np.sqrt(2048 / 8), j
        assert abs(td[:, j].std() - sd) < 0.5 * sd, j


@pytest.mark.parametrize("inner", [5, 1])
def test_subset_da_early_rejection_keeps_the_chains(cuda, inner):
    """Early rejection of the first-stage (coarse-model) moves, of the exact corrections and
    of the plain stages: a CDM delayed-acceptance run with it ends where the run without it
    ends, bit for bit (inner 5: surrogate transitions and an exact correction; inner 1:
    two-stage screening of every step)."""
    from gpu_helpers import cdm_los_oracle, cdm_prior_rows
    from altar_gb300.models import CDM
    g = np.linspace(-20e3, 20e3, 48)
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
        da = DelayedAcceptance(surrogate=SubsetSurrogate(strides=(8, 4)), delta_limit=1.0, check_chains=128,
                               inner=inner, outer=2, stop_beta=1.0, early_reject=early)
        app = Application(model, job=Job(chains=1024, steps=5), rng=RNG(4), controller=Annealer(sampler=da))
        app.initialize()
        app.controller.posterior(model, max_stages=12)
        w = app.controller.worker
        out[early] = ([t.cpu().numpy() for t in (w.step.theta, w.step.data, w.step.posterior)],
                      [(r.get("mode"), r["accepted"], r["rejected"]) for r in w.reports])
    assert any(m == "da" for m, _, _ in out[True][1])
    for a, b in zip(out[False][0], out[True][0]):
        np.testing.assert_array_equal(a, b)
    assert out[False][1] == out[True][1]


def test_trained_network_gain(cuda):
    """What training the network gains.  Two-stage delayed acceptance screens every proposal
    with the network's log-likelihood and runs the exact model only on the survivors, so its
    exact cost per accepted move is (exact evaluations) / (accepted moves); plain Metropolis
    evaluates every proposal inside the prior.  On the Mogi workload (measured on a GB300:
    plain 1.65 exact evaluations per accepted move at 57% acceptance; trained network 1.48 at
    51%; the same sampler with the untrained network, no training passes, 1.81 at 37%) the
    trained network saves exact evaluations per accepted move against plain Metropolis, and
    against the untrained network it saves more and keeps far more moves.  (The Mogi walk
    accepts most proposals, so the screen can save at most the rejected ones.)"""
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    rng = np.random.default_rng(0)
    d = catmip.mogi_los(np.array([[0.0, 0.0, 3e3, 2e6]]), X, Y, los, 0.25, log_strength=False)[0]
    d = d + rng.normal(0, 5e-3, X.size)

    def run(sampler):
        psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 8e3))),
                 "source": Contiguous(1, Uniform((1e5, 1e7)))}
        model = Mogi(psets, observations=Observations(X, Y, los, d, 2.5e-5), log_strength=False)
        app = Application(model, job=Job(chains=2048, steps=5), rng=RNG(7), controller=Annealer(sampler=sampler))
        app.run()
        return app.controller.worker.reports

    def da(epochs):
        sur = Surrogate((4, 128, 128, 32), seed=2, batch=512, lr=2e-3)
        return DelayedAcceptance(surrogate=sur, rms_limit=1e9, delta_limit=float("inf"), fit_chains=1024,
                                 check_chains=128, epochs=epochs, refit_epochs=epochs, inner=1, outer=None,
                                 stop_beta=1.0)

    def figures(reps, mode=None):
        sel = [r for r in reps if mode is None or r.get("mode") == mode]
        acc = sum(r["accepted"] for r in sel)
        prop = sum(r["accepted"] + r["rejected"] + r["unlikely"] for r in sel)
        exact = sum(r["screened"] for r in sel) if mode else sum(r["accepted"] + r["unlikely"] for r in sel)
        return exact / max(acc, 1), acc / max(prop, 1), len(sel)

    plain = figures(run(None))
    trained = figures(run(da(20)), "da")
    untrained = figures(run(da(0)), "da")
    print(f"\nexact evaluations per accepted move / acceptance / stages: plain {plain[0]:.2f} / {plain[1]:.3f} / "
          f"{plain[2]}, trained {trained[0]:.2f} / {trained[1]:.3f} / {trained[2]}, untrained {untrained[0]:.2f} / "
          f"{untrained[1]:.3f} / {untrained[2]}")
    assert trained[2] > 0 and untrained[2] > 0
    assert trained[0] < 0.95 * plain[0]                 # fewer exact evaluations per useful move
    assert trained[0] < 0.9 * untrained[0]
    assert trained[1] > 0.8 * plain[1]                  # most of plain's acceptance kept
    assert trained[1] > 1.2 * untrained[1]              # without training the screen discards good moves


@pytest.mark.parametrize("sizes,n", [(SIZES, 1000), (SIZES, 32768), ((10, 64, 128, 64), 300)])
def test_mlp_forward_tensor_cores(cuda, sizes, n):
    """The tcgen05 forward (split-BF16 activations against the BF16 weights, FP32
    accumulation) against the FP64 oracle with the same BF16-rounded weights, within the
    SIMT forward's tolerance (1e-4 normwise), with and without the FP32 activations kept;
    row counts that are not multiples of the 128-row tile included."""
    sur = Surrogate(sizes, seed=5).init_params()
    assert sur.tc
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (n, sizes[0]))
    lib = _native.load()
    net = ctypes.byref(sur.net)
    xd = dev(x, torch.float32)
    out = torch.empty(n, sizes[-1], dtype=torch.float32, device="cuda")
    acts = torch.empty(lib.ag_mlp_activation_floats(net, n), dtype=torch.float32, device="cuda")
    ws = torch.empty(lib.ag_mlp_tc_workspace_bytes(net, n), dtype=torch.uint8, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    s = stream_handle()
    flat = sur.params.cpu().numpy().astype(np.float64)
    P, o = [], 0
    for fi, fo in zip(sizes[:-1], sizes[1:]):
        W = _bf16_round(flat[o:o + fo * fi].reshape(fo, fi)); o += fo * fi
        P.append((W, flat[o:o + fo])); o += fo
    ref, cache = mlp.forward(P, xd.double().cpu().numpy())
    for keep in (None, acts):
        out.zero_()
        _native.call("ag_mlp_forward_tc", net, ptr(sur.params), ptr(sur.wpack), ptr(xd), n, ptr(out), ptr(keep),
                     ptr(ws), ws.numel(), ptr(flags), s)
        torch.cuda.synchronize()
        assert int(flags.item()) == 0
        got = out.double().cpu().numpy()
        assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref)), np.max(np.abs(got - ref))
    # the kept activations: layer 0's pre-activation and output as the SIMT forward stores them
    z0 = acts[:n * sizes[1]].double().cpu().numpy().reshape(n, sizes[1])
    y0 = acts[n * sizes[1]:2 * n * sizes[1]].double().cpu().numpy().reshape(n, sizes[1])
    assert np.max(np.abs(z0 - cache[0][1])) <= 1e-4 * np.max(np.abs(cache[0][1]))
    assert np.max(np.abs(y0 - mlp.gelu(cache[0][1]))) <= 1e-4 * np.max(np.abs(cache[0][1]))
