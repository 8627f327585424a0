"""Forward models + misfit on the GPU against the oracle and the reference fixtures.

Tolerances (FP32 device arithmetic against FP64 references):
  * CDM LOS displacement, per source, normwise: |u_gpu - u_ref|_inf <= 1e-5 |u_ref|_inf
    for every source (the accuracy bound of the forward model), whatever the angle of its
    sides and its depth.  Rectangles whose sides would cancel (deep relative to their size) are
    integrated by quadrature of point tensile dislocations; near shallow vertices each
    station takes the configuration whose legs point away from it; near-vertical sides are
    evaluated from cancellation-free remainders.  Host build of the same arithmetic: 1,300
    prior sources, max 2.5e-6, median 3e-7; GB300: 300 sources, max 3.4e-6.  The median
    over sources must stay below TOL_CDM_MEDIAN.
  * Mogi LOS displacement: normwise 1e-5.
  * log-likelihood given the device's own FP32 residuals: 1e-9 relative (FP64 oracle sum).
"""
import os

import numpy as np
import pytest
import torch

from altar_gb300 import _native
from oracle import catmip

from gpu_helpers import (LOS, cdm_los_oracle, cdm_prior_rows, cdm_strategy, dev, min_vertical_angle,
                         mogi_strategy)

pytestmark = pytest.mark.gpu

TOL_CDM = 1e-5
TOL_CDM_MEDIAN = 1e-6
G = np.load(os.path.join(os.path.dirname(__file__), "golden", "cdm_golden.npz"))


def _residuals(strategy, theta, m):
    n = theta.shape[0]
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    res = torch.zeros(n, strategy.stations.m_padded, dtype=torch.float32, device="cuda")
    strategy.forward(dev(theta), out, residuals=res)
    torch.cuda.synchronize()
    return out.cpu().numpy(), res.cpu().numpy()[:, :m]


def _fixture_theta():
    # fixture rows: x, y, depth, ax, ay, az, ωx, ωy, ωz, opening, ν
    s = G["ref_src"]
    return np.stack([s[:, 0], s[:, 1], s[:, 2], s[:, 9], s[:, 3], s[:, 4], s[:, 5], s[:, 6], s[:, 7],
                     s[:, 8]], 1)


def test_cdm_matches_reference_fixtures(cuda):
    X, Y = G["ref_X"], G["ref_Y"]
    los = np.tile(LOS, (X.size, 1))
    theta = _fixture_theta()
    strat, _ = cdm_strategy(X, Y, los, np.zeros(X.size), np.full(X.size, 9e-6))
    _, res = _residuals(strat, theta, X.size)
    errs = []
    for k, u in enumerate(G["ref_u"]):
        ref = u[0] * LOS[0] + u[1] * LOS[1] + u[2] * LOS[2]
        err = np.max(np.abs(res[k] - ref)) / np.max(np.abs(ref))
        assert err <= TOL_CDM, (k, err)
        errs.append(err)
    assert np.median(errs) <= TOL_CDM_MEDIAN


def test_cdm_matlab_goldens(cuda):
    """Matlab test source at the 12 golden points (models/cdm/tests/libcdm.py:27-46)."""
    X, Y = G["matlab_X"] * 1e3, G["matlab_Y"] * 1e3        # km -> m keeps FP32 in range
    s = G["matlab_src"]
    th = np.array([[s[0] * 1e3, s[1] * 1e3, s[2] * 1e3, s[9] * 1e3, s[3] * 1e3, s[4] * 1e3, s[5] * 1e3,
                    s[6], s[7], s[8]]])
    for comp, los in (("matlab_ue", [1.0, 0, 0]), ("matlab_un", [0, 1.0, 0]), ("matlab_uv", [0, 0, 1.0])):
        strat, _ = cdm_strategy(X, Y, np.tile(los, (12, 1)), np.zeros(12), np.ones(12))
        _, res = _residuals(strat, th, 12)
        ref = G[comp] * 1e3                                 # displacement scales with length
        # the Matlab source's body z axis is ~9° from the vertical: near-vertical sides
        assert np.max(np.abs(res[0] - ref)) <= TOL_CDM * np.max(np.abs(ref)), comp


def test_cdm_prior_sources_workload_grid(cuda):
    """300 prior sources on an 80 x 80 grid over ±20 km against the FP64 oracle; prints
    the error by the smallest angle between a side and the vertical (run with -s)."""
    g = np.linspace(-20e3, 20e3, 80)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(300, seed=5)
    ref = cdm_los_oracle(theta, X, Y, los)
    strat, _ = cdm_strategy(X, Y, los, np.zeros(X.size), np.full(X.size, 9e-6))
    _, res = _residuals(strat, theta, X.size)
    errs = np.max(np.abs(res - ref), 1) / np.max(np.abs(ref), 1)
    ang = np.array([min_vertical_angle(t) for t in theta])
    print(f"\nCDM normwise error over {len(theta)} prior sources: median {np.median(errs):.2e}, "
          f"max {errs.max():.2e}")
    assert np.all(errs <= TOL_CDM), [(e, a) for e, a in zip(errs, ang) if e > TOL_CDM]
    assert np.median(errs) <= TOL_CDM_MEDIAN
    for lo, hi in ((10, 91), (5, 10), (2, 5), (0, 2)):
        s = (ang >= lo) & (ang < hi)
        if s.any():
            print(f"  smallest side angle [{lo}, {hi}) deg: {s.sum()} sources, median {np.median(errs[s]):.2e}, "
                  f"max {errs[s].max():.2e}")


def test_cdm_work_count_matches_host_plan(cuda):
    """ag_cdm_work (the roofline's FLOP count) follows the likelihood kernel's plan tile by
    tile: against the host build of that plan over the same tile boxes (ag_station_boxes),
    and 0 for a source above the surface.  On the workload's grid the far tiles integrate
    most rectangles with a few nodes, below the work of the chain plan alone."""
    import ctypes
    import shutil
    import subprocess
    import tempfile
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    so = os.path.join(tempfile.mkdtemp(), "cdm_host.so")
    here = os.path.dirname(os.path.abspath(__file__))
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    os.path.join(here, "cdm_host", "cdm_host.cpp"), "-o", so], check=True)
    host = ctypes.CDLL(so)
    P = ctypes.POINTER
    host.cdm_host_plan.argtypes = [P(ctypes.c_double), ctypes.c_double, P(ctypes.c_float), ctypes.c_int,
                                   P(ctypes.c_uint32), P(ctypes.c_int), P(ctypes.c_double), P(ctypes.c_double)]
    theta = cdm_prior_rows(200, seed=31)
    theta = np.concatenate([theta, [[0, 0, 200.0, 1.0, 2000, 2000, 2000, 0, 0, 0]]])
    g = np.linspace(-20e3, 20e3, 200)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    strat, _ = cdm_strategy(X, Y, np.tile(LOS, (X.size, 1)), np.zeros(X.size), np.ones(X.size))
    flop, sfu = strat.work(dev(theta))
    flop = flop.cpu().numpy()
    box = np.ascontiguousarray(strat.stations.tile_box.cpu().numpy())
    assert flop[-1] == 0
    chain_only = []
    for k, th in enumerate(theta[:-1]):
        mask, f, u = ctypes.c_uint32(), ctypes.c_double(), ctypes.c_double()
        nq = (ctypes.c_int * 6)()
        t = np.ascontiguousarray(th)
        assert host.cdm_host_plan(t.ctypes.data_as(P(ctypes.c_double)), 0.25, box.ctypes.data_as(P(ctypes.c_float)),
                                  X.size, ctypes.byref(mask), nq, ctypes.byref(f), ctypes.byref(u)) == 0
        assert flop[k] == f.value, k
        # the chain plan alone: every tile as close as the source centre
        b0 = np.array([[th[0], th[0], th[1], th[1]]], dtype=np.float32)
        assert host.cdm_host_plan(t.ctypes.data_as(P(ctypes.c_double)), 0.25, b0.ctypes.data_as(P(ctypes.c_float)),
                                  1, ctypes.byref(mask), nq, ctypes.byref(f), ctypes.byref(u)) == 0
        chain_only.append(f.value * X.size)
    ratio = np.sum(chain_only) / np.sum(flop[:-1])
    print(f"\nwork of the chain plan / work of the tile plan on the 40,000-station grid: {ratio:.2f}")
    assert ratio > 1.2


def test_cdm_station_order_and_tile_boxes(cuda):
    """The CDM stores its stations along a Hilbert curve: every tile box
    (ag_station_boxes) contains its stations, and the residual rows come back in the
    caller's order, equal (to the quadrature tolerance and FP32 rounding) to those of the
    same stations stored in the caller's order, whose tiles are row segments."""
    from altar_gb300.device import Stations
    rng = np.random.default_rng(17)
    X, Y = rng.uniform(-2e4, 2e4, 3000), rng.uniform(-2e4, 2e4, 3000)
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(40, seed=19)
    d = rng.normal(0, 3e-3, X.size)
    strat, _ = cdm_strategy(X, Y, los, d, np.full(X.size, 9e-6))
    st = strat.stations
    assert st.order is not None
    order = st.order.cpu().numpy()
    assert sorted(order) == list(range(st.m_padded)) and np.all(order[X.size:] == np.arange(X.size, st.m_padded))
    box = st.tile_box.cpu().numpy().astype(np.float64)
    xs, ys = X[order[:X.size]], Y[order[:X.size]]
    for t in range(box.shape[0]):
        sl = slice(128 * t, min(X.size, 128 * (t + 1)))
        assert box[t, 0] <= xs[sl].min() and xs[sl].max() <= box[t, 1], t
        assert box[t, 2] <= ys[sl].min() and ys[sl].max() <= box[t, 3], t
    llk, res = _residuals(strat, theta, X.size)
    # the same stations stored in the caller's order
    strat.stations = Stations(X, Y, los, d, np.full(X.size, 1 / 9e-6), reorder=False)
    llk0, res0 = _residuals(strat, theta, X.size)
    err = np.max(np.abs(res - res0), 1) / np.max(np.abs(res0 + d), 1)
    assert err.max() < 2e-6, err.max()
    np.testing.assert_allclose(llk, llk0, rtol=1e-6)
    ref = cdm_los_oracle(theta[:8], X, Y, los)
    assert np.max(np.abs(res[:8] + d - ref)) <= TOL_CDM * np.max(np.abs(ref))


def test_cdm_launch_variants_identical(cuda):
    """Every launch variant (warps per CTA, register budget, one, two or four stations per
    lane) computes the same residuals and log-likelihoods bit for bit: the rounding of every
    operation is fixed in the source and each lane accumulates its stations in one order."""
    lib = _native.load()
    g = np.linspace(-20e3, 20e3, 200)[::4]
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(37, seed=12)
    d = np.random.default_rng(1).normal(0, 3e-3, X.size)
    runs = {}
    for v in range(lib.ag_forward_variants(_native.AG_MODEL_CDM)):
        strat, _ = cdm_strategy(X, Y, los, d, np.full(X.size, 9e-6), variant=v)
        runs[v] = _residuals(strat, theta, X.size)
    llk0, res0 = runs[0]
    ref = cdm_los_oracle(theta[:4], X, Y, los)
    assert np.max(np.abs(res0[:4] + d - ref)) <= 1e-3 * np.max(np.abs(ref))
    for v, (llk, res) in runs.items():
        np.testing.assert_array_equal(res, res0, err_msg=f"variant {v}")
        np.testing.assert_array_equal(llk, llk0, err_msg=f"variant {v}")


def test_cdm_degenerate_axes(cuda):
    """The reference's special cases (libcdm.py:226-242): one zero semi-axis leaves a single
    rectangle, all three zero give no displacement; a rotation by 0 makes four sides
    exactly vertical, which contribute nothing (libcdm.py:320-324)."""
    g = np.linspace(-20e3, 20e3, 200)[::8]
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    # x, y, depth, opening, ax, ay, az, ωx, ωy, ωz
    theta = np.array([
        [1e3, -2e3, 5e3, 10.0, 0.0, 1500.0, 800.0, 20.0, -35.0, 60.0],     # ax = 0
        [1e3, -2e3, 5e3, 10.0, 1200.0, 0.0, 800.0, 20.0, -35.0, 60.0],     # ay = 0
        [1e3, -2e3, 5e3, 10.0, 1200.0, 1500.0, 0.0, 20.0, -35.0, 60.0],    # az = 0
        [1e3, -2e3, 5e3, 10.0, 0.0, 0.0, 0.0, 20.0, -35.0, 60.0],          # point: no displacement
        [-3e3, 4e3, 6e3, -8.0, 900.0, 1100.0, 700.0, 0.0, 0.0, 30.0],      # vertical sides
    ])
    strat, _ = cdm_strategy(X, Y, los, np.zeros(X.size), np.full(X.size, 9e-6))
    _, res = _residuals(strat, theta, X.size)
    ref = cdm_los_oracle(theta, X, Y, los)
    assert np.all(res[3] == 0.0) and np.all(ref[3] == 0.0)
    for k in (0, 1, 2, 4):
        err = np.max(np.abs(res[k] - ref[k])) / np.max(np.abs(ref[k]))
        assert err <= TOL_CDM, (k, err)


def test_cdm_llk_given_residuals(cuda):
    rng = np.random.default_rng(2)
    g = np.linspace(-20e3, 20e3, 40)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(32, seed=5)
    truth = cdm_los_oracle(theta[:1], X, Y, los)[0]
    d = truth + rng.normal(0, 3e-3, X.size)
    var = np.full(X.size, 9e-6)
    strat, obs = cdm_strategy(X, Y, los, d, var)
    llk, res = _residuals(strat, theta, X.size)
    w = np.full(X.size, np.float32(1.0 / 9e-6), dtype=np.float64)
    ref = catmip.llk_from_residuals(res.astype(np.float64), w, obs.normalization())
    assert np.max(np.abs(llk - ref) / np.abs(ref)) < 1e-9
    # end to end against the FP64 oracle: bounded by the FP32 forward error
    full, _ = catmip.diag_llk(cdm_los_oracle(theta, X, Y, los), d, var)
    rel = np.abs(llk - full) / np.abs(full)
    assert np.median(rel) < 1e-6 and rel.max() < 1e-5, (np.median(rel), rel.max())


def test_cdm_mask_and_surface_status(cuda):
    g = np.linspace(-5e3, 5e3, 10)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    theta = cdm_prior_rows(4, seed=9)
    theta[1, 2] = 200.0          # shallow and large: above the surface
    theta[1, 4:7] = 2000.0
    strat, _ = cdm_strategy(X, Y, los, np.zeros(X.size), np.ones(X.size))
    out = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    mask = torch.tensor([0, 0, 1, 0], dtype=torch.int32, device="cuda")
    strat.forward(dev(theta), out, mask=mask, status=mask)
    torch.cuda.synchronize()
    m = mask.cpu().numpy()
    o = out.cpu().numpy()
    assert m[1] & _native.AG_CHAIN_ABOVE_SURFACE and m[2] == 1 and m[0] == 0 and m[3] == 0
    assert o[1] == 7.0 and o[2] == 7.0 and o[0] != 7.0 and o[3] != 7.0


def test_cdm_dataset_offsets(cuda):
    """Per-dataset offsets θ[offset_idx + oid] (cdm/Native.py:225-227)."""
    g = np.linspace(-10e3, 10e3, 12)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    oid = (X > 0).astype(np.int32)
    base = cdm_prior_rows(3, seed=4)
    theta = np.concatenate([base, np.array([[0.01, -0.02]] * 3)], 1)
    d = np.zeros(X.size)
    strat, obs = cdm_strategy(X, Y, los, d, np.full(X.size, 1e-4), oid=oid, offset_idx=10, nparams=12)
    llk, res = _residuals(strat, theta, X.size)
    ref = cdm_los_oracle(base, X, Y, los) - theta[:, 10 + oid]
    assert np.max(np.abs(res - ref)) <= 1e-4 * np.max(np.abs(ref))


def test_mogi_matches_oracle(cuda):
    rng = np.random.default_rng(1)
    X, Y = rng.uniform(-25e3, 25e3, 3000), rng.uniform(-25e3, 25e3, 3000)
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    theta = np.stack([rng.uniform(-1e4, 1e4, 100), rng.uniform(-1e4, 1e4, 100), rng.uniform(1e3, 8e3, 100),
                      rng.uniform(1e5, 1e7, 100)], 1)
    d = catmip.mogi_los(theta[:1], X, Y, los, 0.25, log_strength=False)[0] + rng.normal(0, 5e-3, X.size)
    var = np.full(X.size, 2.5e-5)
    strat, obs = mogi_strategy(X, Y, los, d, var)
    llk, res = _residuals(strat, theta, X.size)
    ref_u = catmip.mogi_los(theta, X, Y, los, 0.25, log_strength=False)
    err = np.max(np.abs((res + d) - ref_u), 1) / np.max(np.abs(ref_u), 1)
    assert np.all(err < 1e-5), err.max()
    w = np.full(X.size, np.float32(1 / 2.5e-5), dtype=np.float64)
    ref = catmip.llk_from_residuals(res.astype(np.float64), w, obs.normalization())
    assert np.max(np.abs(llk - ref) / np.abs(ref)) < 1e-9


def test_mogi_two_sources_log_strength(cuda):
    rng = np.random.default_rng(3)
    X, Y = rng.uniform(-25e3, 25e3, 500), rng.uniform(-25e3, 25e3, 500)
    los = np.tile([0.1, 0.5, 0.86], (X.size, 1))
    # two sources, [x, y, depth, log10 ΔV] each, stride 4
    theta = np.stack([rng.uniform(-1e4, 1e4, 20), rng.uniform(-1e4, 1e4, 20), rng.uniform(1e3, 8e3, 20),
                      rng.uniform(5, 7, 20), rng.uniform(-1e4, 1e4, 20), rng.uniform(-1e4, 1e4, 20),
                      rng.uniform(1e3, 8e3, 20), rng.uniform(5, 7, 20)], 1)
    strat, obs = mogi_strategy(X, Y, los, np.zeros(X.size), np.ones(X.size), log_strength=True, nparams=8,
                               nsources=2, stride=4)
    _, res = _residuals(strat, theta, X.size)
    ref = catmip.mogi_los(theta, X, Y, los, 0.25, log_strength=True, nsources=2, stride=4)
    err = np.max(np.abs(res - ref), 1) / np.max(np.abs(ref), 1)
    assert np.all(err < 1e-5), err.max()


@pytest.mark.parametrize("nsources", [1, 2])
def test_mogi_launch_variants_identical(cuda, nsources):
    """The Mogi launch variants (8, 16 or 32 chains per CTA) differ only in how many chains a
    CTA holds: each lane accumulates the same stations in the same order, so residuals and
    log-likelihoods agree bit for bit; the autotuner picks among them."""
    lib = _native.load()
    assert lib.ag_forward_variants(_native.AG_MODEL_MOGI) == 3
    rng = np.random.default_rng(11)
    X, Y = rng.uniform(-25e3, 25e3, 1000), rng.uniform(-25e3, 25e3, 1000)
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    cols = [rng.uniform(-1e4, 1e4, 77), rng.uniform(-1e4, 1e4, 77), rng.uniform(1e3, 8e3, 77),
            rng.uniform(5, 7, 77)]
    theta = np.stack(cols * nsources, 1)
    d = rng.normal(0, 5e-3, X.size)
    runs = {}
    for v in range(3):
        strat, _ = mogi_strategy(X, Y, los, d, np.full(X.size, 2.5e-5), log_strength=True,
                                 nparams=4 * nsources, nsources=nsources, stride=4 if nsources > 1 else 0)
        strat.layout.variant = v
        runs[v] = _residuals(strat, theta, X.size)
    llk0, res0 = runs[0]
    for v, (llk, res) in runs.items():
        np.testing.assert_array_equal(res, res0, err_msg=f"variant {v}")
        np.testing.assert_array_equal(llk, llk0, err_msg=f"variant {v}")


def test_host_buffer_call_pattern(cuda):
    """The reference's call pattern: host θ in, host data log-likelihood out."""
    rng = np.random.default_rng(8)
    X, Y = rng.uniform(-15e3, 15e3, 256), rng.uniform(-15e3, 15e3, 256)
    los = np.tile([0.38, -0.08, 0.92], (X.size, 1))
    strat, _ = mogi_strategy(X, Y, los, np.zeros(X.size), np.ones(X.size))
    theta = np.stack([rng.uniform(-1e4, 1e4, 10), rng.uniform(-1e4, 1e4, 10), rng.uniform(1e3, 8e3, 10),
                      rng.uniform(1e5, 1e7, 10)], 1)

    class Step:
        pass

    step = Step()
    step.theta = theta
    step.data = np.zeros(10)
    strat.dataLikelihood(None, step)
    out = torch.empty(10, dtype=torch.float64, device="cuda")
    strat.forward(dev(theta), out)
    np.testing.assert_array_equal(step.data, out.cpu().numpy())


def test_cdm_dense_cd_from_case_files(cuda, tmp_path):
    """A case directory with a dense cd.txt (models/cdm/cdm/CDM.py:275-355): the reader keeps
    Cd dense, the fused kernel writes residual rows and the tcgen05 whitening adds
    -1/2 rᵀ Cd⁻¹ r.  Checked against FP64: (1) given the kernel's own FP32 residual rows,
    llk = -1/2 (M log 2π + log det Cd + rᵀ Cd⁻¹ r) within 1e-5 relative + 0.05 for a population
    near the truth and 1e-4 relative for prior draws (the split-BF16 whitening, as the linear
    model's tests); (2) end to end for prior draws within 1e-4 relative.  Near the
    truth the misfit is small and the FP32 forward error (~3e-6 of the field) amplified by
    L⁻¹ dominates the end-to-end difference, so those chains are held to (1)."""
    import math

    from altar_gb300.models.forward import CUDA
    from altar_gb300.models.observations import Observations
    from gpu_helpers import Shim
    from test_observations_cpu import write_case

    rng = np.random.default_rng(4)
    m = 300
    x, y = rng.uniform(-2e4, 2e4, m), rng.uniform(-2e4, 2e4, m)
    th_los, ph_los = np.full(m, 0.4), np.full(m, -1.2)
    los = np.stack([np.sin(th_los) * np.cos(ph_los), np.sin(th_los) * np.sin(ph_los), np.cos(th_los)], 1)
    dist = np.hypot(x[:, None] - x[None, :], y[:, None] - y[None, :])
    cd = 9e-6 * (0.8 * np.exp(-dist / 2e3) + 0.2 * np.eye(m))
    truth = cdm_prior_rows(1, seed=40)
    d = cdm_los_oracle(truth, x, y, los)[0] + np.linalg.cholesky(cd) @ rng.normal(size=m)
    write_case(tmp_path, x, y, d, th_los, ph_los, cd)
    obs = Observations.read(str(tmp_path))
    assert obs.dense
    lay = _native.Layout(10, 0, 2, 3, 4, 7, -1, 0, 1, 0, nu=0.25)
    strat = CUDA(_native.AG_MODEL_CDM).initialize(None, Shim(obs, lay))
    near = truth + rng.normal(size=(32, 10)) * [50, 50, 50, 0.5, 20, 20, 20, 1, 1, 1]
    prior = cdm_prior_rows(32, seed=41)
    sign, logdet = np.linalg.slogdet(cd)
    norm = -0.5 * (m * math.log(2 * math.pi) + logdet)

    def llk(r):
        return norm - 0.5 * np.einsum("ij,ji->i", r, np.linalg.solve(cd, r.T))

    # one population per call, as the sampler evaluates them (the whitening centres the residual
    # rows on the population's mean before the split-BF16 product)
    for theta, rel_given, abs_given in ((near, 1e-5, 0.05), (prior, 1e-4, 0.0)):
        out = torch.empty(theta.shape[0], dtype=torch.float64, device="cuda")
        res = torch.zeros(theta.shape[0], strat.stations.m_padded, dtype=torch.float32, device="cuda")
        strat.forward(dev(theta), out, residuals=res)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        given = llk(res.cpu().numpy()[:, :m].astype(np.float64))
        assert np.all(np.abs(got - given) <= rel_given * np.abs(given) + abs_given), \
            np.max(np.abs(got - given) / np.abs(given))
    e2e = llk(cdm_los_oracle(prior, x, y, los) - d[None, :])
    rel = np.abs(got - e2e) / np.abs(e2e)
    assert np.all(rel <= 1e-4), rel.max()
