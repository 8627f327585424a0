"""Equal-posterior statistics of the sampler sweep (bench.equal_posterior), on the CPU.

The sweep decides which plain walk is the cheapest one that reaches the converged
posterior and whether delayed acceptance reaches it: runs in a secondary mode are set
apart, then each summary's seed mean is compared with the reference sampler's in units
of the combined standard error.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _run(mean, llk=0.0, t=1.0, stages=40):
    return {"time_s": t, "stages": stages, "llk_max": llk, "invariants": {"mean": list(mean)}}


def _sampler(rng, centre, spread, k, llk=0.0, t=1.0):
    return [_run(centre + spread * rng.standard_normal(len(centre)), llk=llk, t=t) for _ in range(k)]


def test_z_scores_match_the_formula():
    rng = np.random.default_rng(3)
    ref = _sampler(rng, np.zeros(3), 1.0, 5)
    other = _sampler(rng, np.array([0.5, -0.2, 0.0]), 2.0, 4)
    out = bench.equal_posterior({"plain20": ref, "da": other}, "plain20")
    a = np.array([r["invariants"]["mean"] for r in other])
    b = np.array([r["invariants"]["mean"] for r in ref])
    z = (a.mean(0) - b.mean(0)) / np.sqrt(a.var(0, ddof=1) / 4 + b.var(0, ddof=1) / 5)
    np.testing.assert_allclose(out["da"]["z"], z, rtol=1e-12)
    np.testing.assert_allclose(out["plain20"]["z"], 0.0, atol=0.0)
    assert out["plain20"]["reaches"]


def test_recorded_sweep_z():
    """The x and a_max summaries of the five-seed sweep of the 20-step walk against
    delayed acceptance with 20 first-stage moves (z 1.4508 and 0.5604 as recorded)."""
    ref_x = [3516.415540055, 3516.4185830257, 3516.4312774625, 3516.4149733833, 3516.4177248171]
    ref_a = [2987.4730951823, 2987.4703665712, 2987.4775946405, 2987.4706843825, 2987.472091175]
    ref_l = [175866.83969757363, 175867.05415358403, 175866.85727410455, 175867.06338605407, 175866.89642103214]
    da_x = [3516.4173427762, 3516.4357803113, 3516.4434993417, 3516.4145891466, 3516.4971838056]
    da_a = [2987.4894745294, 2987.4541677992, 2987.4734564736, 2987.4725580295, 2987.4944551733]
    da_l = [175867.0542259249, 175866.71227989724, 175866.86370603542, 175866.86617611969, 175866.95896738436]
    runs = {"plain20": [_run([x, a], llk=l) for x, a, l in zip(ref_x, ref_a, ref_l)],
            "da": [_run([x, a], llk=l) for x, a, l in zip(da_x, da_a, da_l)]}
    out = bench.equal_posterior(runs, "plain20")
    np.testing.assert_allclose(out["da"]["z"], [1.4508000378260082, 0.5603950941690732], rtol=1e-8)
    assert out["da"]["trapped_runs"] == 0 and out["da"]["reaches"]


def test_trapped_runs_are_set_apart():
    """A run 13,580 below the others (a secondary mode) leaves the summaries and counts
    against its sampler; with the reference free of such runs that sampler fails."""
    rng = np.random.default_rng(5)
    ref = _sampler(rng, np.zeros(2), 1.0, 5, llk=100.0)
    good = _sampler(rng, np.zeros(2), 1.0, 4, llk=100.0)
    trapped = good + [_run([500.0, -500.0], llk=100.0 - 13580.0)]
    out = bench.equal_posterior({"plain20": ref, "plain10": trapped, "da": good}, "plain20")
    assert out["plain10"]["trapped_runs"] == 1 and not out["plain10"]["reaches"]
    # the trapped run's summary does not enter the z-scores
    np.testing.assert_allclose(out["plain10"]["z"], out["da"]["z"], rtol=1e-12)
    assert out["da"]["reaches"]
    # its time still counts in the sampler's mean
    assert len(out["plain10"]["times_s"]) == 5


def test_trap_threshold():
    rng = np.random.default_rng(6)
    ref = _sampler(rng, np.zeros(2), 1.0, 4, llk=0.0)
    near = _sampler(rng, np.zeros(2), 1.0, 3, llk=0.0) + [_run([0.1, 0.1], llk=-bench.TRAP_LLK)]
    far = _sampler(rng, np.zeros(2), 1.0, 3, llk=0.0) + [_run([0.1, 0.1], llk=-bench.TRAP_LLK - 1e-6)]
    out = bench.equal_posterior({"ref": ref, "near": near, "far": far}, "ref")
    assert out["near"]["trapped_runs"] == 0
    assert out["far"]["trapped_runs"] == 1


def test_shifted_sampler_fails():
    """A sampler whose seed mean sits 3 combined standard errors off the reference fails."""
    base = np.array([-1.0, 0.0, 1.0, 0.5, -0.5])
    ref = [_run([v, 0.0]) for v in base]
    sd = base.std(ddof=1)
    se = np.sqrt(2 * sd ** 2 / 5)
    off = [_run([v + 3.0 * se, 0.0]) for v in base]
    near = [_run([v + 1.5 * se, 0.0]) for v in base]
    out = bench.equal_posterior({"ref": ref, "off": off, "near": near}, "ref")
    assert out["off"]["z"][0] == pytest.approx(3.0) and not out["off"]["reaches"]
    assert out["near"]["z"][0] == pytest.approx(1.5) and out["near"]["reaches"]


def test_one_run_cannot_reach():
    rng = np.random.default_rng(8)
    ref = _sampler(rng, np.zeros(2), 1.0, 5)
    out = bench.equal_posterior({"ref": ref, "one": [_run([0.0, 0.0])]}, "ref")
    assert not out["one"]["reaches"]


def test_every_run_trapped():
    rng = np.random.default_rng(9)
    ref = _sampler(rng, np.zeros(2), 1.0, 5, llk=0.0)
    lost = [_run([3.0, 3.0], llk=-1e4) for _ in range(3)]
    out = bench.equal_posterior({"ref": ref, "lost": lost}, "ref")
    assert out["lost"]["trapped_runs"] == 3 and not out["lost"]["reaches"]


def test_sweep_line_with_several_da_settings(monkeypatch, capsys):
    """run_sweep with stand-in runs: the first delayed-acceptance setting is the line's
    "da"; every setting gets its time, whether it reaches the reference posterior, and its
    speed-up against the cheapest plain walk that reaches it."""
    import argparse
    import json
    import torch

    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    # every sampler sees the same per-seed scatter; the 5-step walk is shifted off it
    scatter = dict(zip([1, 2, 3, 4, 5], np.random.default_rng(11).standard_normal((5, 7))))

    def fake_anneal(kind, X, Y, los, d, N, rank, args, seed=1234, max_stages=None):
        if kind == "plain":
            t, shift = 2.0 * args.walk_steps, (4.0 if args.walk_steps == 5 else 0.0)
        else:
            t, shift = float(args.da_inner) / 2, 0.0
        mean = shift + scatter.get(seed, np.zeros(7))
        return {"time_s": t, "stages": 40, "llk_max": 0.0,
                "invariants": {"mean": mean.tolist(), "names": list("abcdefg")}}

    monkeypatch.setattr(bench, "anneal", fake_anneal)
    args = argparse.Namespace(seeds=[1, 2, 3, 4, 5], sweep_steps=[5, 15, 20], sweep_da=["20x1", "10x1"],
                              walk_steps=5)
    assert bench.run_sweep(args, np.zeros(4), np.zeros(4), None, None, 8, 0) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["config"]["reference"] == "plain20"
    assert line["cheapest_plain_at_equal_posterior"] == "plain15"
    assert not line["samplers"]["plain5"]["reaches"]
    assert set(line["da_settings"]) == {"20x1", "10x1"}
    assert line["da_settings"]["20x1"]["key"] == "da" and line["da_settings"]["10x1"]["key"] == "da10x1"
    assert line["value"] == pytest.approx(10.0)
    assert line["speedup_da_vs_plain_at_equal_posterior"] == pytest.approx(30.0 / 10.0)
    assert line["da_settings"]["10x1"]["speedup_vs_cheapest_plain"] == pytest.approx(30.0 / 5.0)
