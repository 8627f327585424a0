"""Posterior summaries of the oracle CATMIP loop over several seeds (test fixtures).

Runs ``oracle.catmip.Annealing`` -- the FP64 restatement of the reference's
annealing loop (altar/altar/bayesian/Annealer.py:79-135 with COV.py:66-251 and
Metropolis.py:63-281) that draws from the same Philox streams as the device --
on two problems for seeds 1..K (8 Mogi, 24 CDM) and stores, per seed, the summaries
of the final population.  Seeds can be generated in batches (--cdm-first-seed,
--cdm-seeds, --skip-mogi) and their rows concatenated in seed order.  The spread of a summary over the seeds is the Monte Carlo standard
error of one run (it includes the correlation the resampling introduces).

  * ``mogi_*``: the Mogi workload (1,024 LOS points on a 32x32 grid over ±15 km,
    LOS (0.38, -0.08, 0.92), truth (0, 0, 3 km, 2e6 m³) + N(0, (5 mm)²) noise,
    priors x, y ~ U[-10, 10] km, depth ~ U[1, 8] km, ΔV ~ U[1e5, 1e7] m³,
    1,024 chains, 5 steps per stage, grid β solver); summaries: mean and sd of
    each parameter.
  * ``cdm_*``: a CDM case on a 24x24 grid over ±20 km (576 stations), a fixed
    truth inside the workload priors + N(0, (3 mm)²) noise, 2,048 chains, 5 steps
    per stage; log-likelihoods from the FP64 C restatement of libcdm.py
    (oracle/csrc/catmip_ref.c); summaries: mean and sd of x, y, depth, opening
    and the per-sample sorted semi-axes (independent of which of the CDM's
    equivalent parameterisations a run settles in).

The station coordinates and data are stored too, so the GPU tests use the very
same inputs.  Run here (CPU):  python tests/golden/make_posterior_golden.py
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import catmip, cdm, cref  # noqa: E402

LOS = np.array([0.38, -0.08, 0.92])
CDM_LO = np.array([-1e4, -1e4, 1e3, -50.0, 100.0, 100.0, 100.0, -90.0, -90.0, -90.0])
CDM_HI = np.array([1e4, 1e4, 1e4, 50.0, 3000.0, 3000.0, 3000.0, 90.0, 90.0, 90.0])
CDM_TRUTH = np.array([1500.0, -2200.0, 4200.0, 18.0, 1400.0, 700.0, 1100.0, 25.0, -40.0, 60.0])


def summaries_mogi(theta):
    return np.concatenate([theta.mean(0), theta.std(0)])


def summaries_cdm(theta):
    q = np.concatenate([theta[:, 0:4], np.sort(theta[:, 4:7], axis=1)], axis=1)
    return np.concatenate([q.mean(0), q.std(0)])


def mogi_case():
    g = np.linspace(-15e3, 15e3, 32)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    truth = np.array([[0.0, 0.0, 3e3, 2e6]])
    d = catmip.mogi_los(truth, X, Y, los, 0.25, log_strength=False)[0] + \
        np.random.default_rng(0).normal(0, 5e-3, X.size)
    return X, Y, d


def cdm_case():
    g = np.linspace(-20e3, 20e3, 24)
    X, Y = [a.ravel() for a in np.meshgrid(g, g)]
    los = np.tile(LOS, (X.size, 1))
    lay = {"x": 0, "depth": 2, "opening": 3, "ax": 4, "omega": 7}
    u = cdm.los_displacements(CDM_TRUTH, lay, X, Y, los, 0.25)
    d = u + np.random.default_rng(1).normal(0, 3e-3, X.size)
    return X, Y, d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=8)
    ap.add_argument("--cdm-seeds", type=int, default=24)
    ap.add_argument("--cdm-first-seed", type=int, default=1)
    ap.add_argument("--skip-mogi", action="store_true")
    ap.add_argument("--out", default=os.path.join(HERE, "posterior_golden.npz"))
    args = ap.parse_args()
    out = {}

    X, Y, d = mogi_case()
    los = np.tile(LOS, (X.size, 1))
    lo, hi = np.array([-1e4, -1e4, 1e3, 1e5]), np.array([1e4, 1e4, 8e3, 1e7])

    def mogi_llk(th):
        u = catmip.mogi_los(th, X, Y, los, 0.25, log_strength=False)
        return catmip.diag_llk(u, d, np.full(X.size, 2.5e-5))[0], np.zeros(th.shape[0], bool)

    rows, stages = [], []
    for seed in range(1, 0 if args.skip_mogi else args.seeds + 1):
        r = catmip.Annealing(mogi_llk, lo, hi, chains=1024, steps=5, seed=seed).run()
        rows.append(summaries_mogi(r["theta"]))
        stages.append(len(r["stages"]))
        print(f"mogi seed {seed}: {len(r['stages'])} stages", flush=True)
    out.update(mogi_X=X, mogi_Y=Y, mogi_d=d, mogi_summaries=np.array(rows), mogi_stages=np.array(stages))

    X, Y, d = cdm_case()
    los = np.tile(LOS, (X.size, 1))
    w = np.full(X.size, 1.0 / 9e-6)
    norm = -0.5 * (X.size * np.log(2 * np.pi) + X.size * np.log(9e-6))
    layout = cref.RefLayout(10, 0, 2, 3, 4, 7, 0, 0.25)

    def cdm_llk(th):
        return cref.llk(2, th, layout, X, Y, los.ravel(), d, w, norm, nthreads=os.cpu_count())

    rows, stages = [], []
    for seed in range(args.cdm_first_seed, args.cdm_first_seed + args.cdm_seeds):
        r = catmip.Annealing(cdm_llk, CDM_LO, CDM_HI, chains=2048, steps=5, seed=seed).run()
        rows.append(summaries_cdm(r["theta"]))
        stages.append(len(r["stages"]))
        print(f"cdm seed {seed}: {len(r['stages'])} stages", flush=True)
    out.update(cdm_X=X, cdm_Y=Y, cdm_d=d, cdm_truth=CDM_TRUTH, cdm_summaries=np.array(rows),
               cdm_stages=np.array(stages))
    np.savez_compressed(args.out, **out)


if __name__ == "__main__":
    main()
