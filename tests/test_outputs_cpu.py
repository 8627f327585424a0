"""Output formats written by the host side (no GPU): the sample layout file."""
import csv

from altar_gb300.distributions import Uniform
from altar_gb300.models import Bayesian, Contiguous


def test_parameters_csv_layout(tmp_path):
    """parameters.csv holds name, count, offset per parameter set, as the reference's
    models write it (models/cdm/cdm/CDM.py:358-380)."""
    psets = {"location": Contiguous(2, Uniform((-1e4, 1e4))), "depth": Contiguous(1, Uniform((1e3, 1e4))),
             "opening": Contiguous(1, Uniform((-50, 50))), "a": Contiguous(3, Uniform((100, 3000))),
             "omega": Contiguous(3, Uniform((-90, 90)))}
    model = Bayesian(psets=psets)
    offset = 0
    for pset in psets.values():
        offset += pset.initialize(model=model, offset=offset)
    path = tmp_path / "parameters.csv"
    model.meta(str(path))
    with open(path, newline="") as f:
        rows = list(csv.reader(f))
    assert rows == [["name", "count", "offset"], ["location", "2", "0"], ["depth", "1", "2"],
                    ["opening", "1", "3"], ["a", "3", "4"], ["omega", "3", "7"]]


class _Clock:
    """Host stand-in for the CUDA-event clock: marks are counters one second apart."""

    def __init__(self):
        self.t = 0.0

    def mark(self):
        self.t += 1.0
        return self.t

    def seconds(self, a, b):
        return b - a


def test_profiler_csv_layout(tmp_path):
    """The profiler's file name and layout follow the reference (altar/altar/bayesian/
    Profiler.py:33-35, 302-362): run characteristics, then the twelve phases with their
    totals.  The events are fired in the order Annealer.posterior fires them."""
    from types import SimpleNamespace

    from altar_gb300.bayesian import Notifier, Profiler

    d = Notifier()
    prof = Profiler(directory=str(tmp_path), clock=_Clock())
    d.register(prof)
    ctl = SimpleNamespace(model=SimpleNamespace(parameters=10, job=SimpleNamespace(chains=512, steps=3)),
                          worker=SimpleNamespace(wid=1))
    ev = lambda name: d.notify(event=getattr(d, name), controller=ctl)
    ev("start")
    for _ in range(4):                                   # four β steps
        ev("betaStart")
        ev("walkChainsStart")
        ev("samplePosteriorStart")
        ev("prepareSamplingPDFStart")
        ev("prepareSamplingPDFFinish")
        for _ in range(3):
            for pair in ("chainAdvance", "verify", "data", "accept"):
                ev(pair + "Start")
            for pair in ("accept", "data", "verify", "chainAdvance"):
                ev(pair + "Finish")
        ev("samplePosteriorFinish")
        ev("walkChainsFinish")
        ev("resampleStart")
        ev("resampleFinish")
        ev("betaFinish")
    ev("finish")
    assert d.start == "simulationStart" and d.finish == "simulationFinish" and d.eager
    name = tmp_path / "prof-00001-004x010x000512x003.csv"
    assert prof.filename == str(name)
    with open(name, newline="") as f:
        rows = list(csv.reader(f))
    assert rows[:6] == [["run characteristics"], ["beta steps", "4"], ["parameters", "10"], ["chains", "512"],
                        ["steps", "3"], ["timings"]]
    phases = [r[0] for r in rows[6:]]
    assert phases == ["simulation", "samplePosterior", "prepareSamplingPDF", "beta", "walk", "chainAdvance",
                      "verify", "prior", "data", "posterior", "accept", "resample"]
    t = {r[0]: float(r[1]) for r in rows[6:]}
    # each accept span is one tick (its finish is the next mark), 12 of them; prior and posterior
    # are fused into the proposal and accept launches inside a walk and never fire here
    assert t["accept"] == 12.0 and t["prior"] == 0.0 and t["posterior"] == 0.0
    assert t["simulation"] > t["beta"] > t["walk"] > t["samplePosterior"] > t["chainAdvance"]
