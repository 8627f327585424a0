"""Event bus and phase profiler (altar/altar/bayesian/Notifier.py:27-83, Profiler.py).

The Notifier carries the reference's event names; the Profiler times the
annealing phases with CUDA events on the annealer's stream and writes a CSV
with one row per stage.
"""
import csv

import torch

EVENTS = ("start", "finish", "betaStart", "betaFinish", "walkChainsStart", "walkChainsFinish",
          "resampleStart", "resampleFinish", "samplePosteriorStart", "samplePosteriorFinish",
          "prepareSamplingPDFStart", "prepareSamplingPDFFinish", "chainAdvanceStart",
          "chainAdvanceFinish", "verifyStart", "verifyFinish", "priorStart", "priorFinish",
          "dataStart", "dataFinish", "posteriorStart", "posteriorFinish", "acceptStart",
          "acceptFinish")


class Notifier:
    def __init__(self):
        for name in EVENTS:
            setattr(self, name, name)
        self.monitors = []

    def initialize(self, application):
        return self

    def register(self, monitor):
        self.monitors.append(monitor)
        return self

    def notify(self, event, controller):
        for m in self.monitors:
            handler = getattr(m, event, None)
            if handler is not None:
                handler(controller=controller)
        return self


class Profiler:
    """Per-stage device time of the cool / walk / resample phases."""

    PHASES = ("beta", "walk", "resample")

    def __init__(self, path=None):
        self.path = path
        self.rows = []
        self._ev = {}

    def initialize(self, application):
        return self

    def _mark(self, key):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        self._ev[key] = ev

    def betaStart(self, controller):
        self._mark("beta0")

    def walkChainsStart(self, controller):
        self._mark("walk0")

    def walkChainsFinish(self, controller):
        self._mark("walk1")

    def resampleStart(self, controller):
        self._mark("res0")

    def betaFinish(self, controller):
        self._mark("res1")
        e = self._ev
        e["res1"].synchronize()
        self.rows.append({
            "stage": len(self.rows),
            "beta": e["beta0"].elapsed_time(e["walk0"]),
            "walk": e["walk0"].elapsed_time(e["walk1"]),
            "resample": e["res0"].elapsed_time(e["res1"]),
        })

    def finish(self, controller):
        if self.path:
            with open(self.path, "w", newline="") as f:
                w = csv.DictWriter(f, fieldnames=["stage", "beta", "walk", "resample"])
                w.writeheader()
                w.writerows(self.rows)
