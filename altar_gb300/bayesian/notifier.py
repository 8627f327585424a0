"""Event bus and phase profiler (altar/altar/bayesian/Notifier.py:20-83, Profiler.py:21-362).

The Notifier carries the reference's event names (``start`` is "simulationStart",
``finish`` "simulationFinish"); monitors register handlers named after the events.
The Profiler accumulates the time of the reference's twelve phases and writes the
reference's CSV file: a run-characteristics block (β steps, parameters, chains,
steps) followed by one row per phase with its total time in seconds, named
``prof-{wid:05}-{beta:03}x{parameters:03}x{chains:06}x{steps:03}.csv``
(Profiler.py:33-35, 302-362).  The times are device times on the annealer's
stream, taken with CUDA events, where the reference reads wall-clock timers.
"""
import csv
import os

EVENTS = {
    "start": "simulationStart", "finish": "simulationFinish",
    "betaStart": "betaStart", "betaFinish": "betaFinish",
    "walkChainsStart": "walkChainsStart", "walkChainsFinish": "walkChainsFinish",
    "resampleStart": "resampleStart", "resampleFinish": "resampleFinish",
    "samplePosteriorStart": "samplePosteriorStart", "samplePosteriorFinish": "samplePosteriorFinish",
    "prepareSamplingPDFStart": "prepareSamplingPDFStart", "prepareSamplingPDFFinish": "prepareSamplingPDFFinish",
    "chainAdvanceStart": "chainAdvanceStart", "chainAdvanceFinish": "chainAdvanceFinish",
    "verifyStart": "verifyStart", "verifyFinish": "verifyFinish",
    "priorStart": "priorStart", "priorFinish": "priorFinish",
    "dataStart": "dataStart", "dataFinish": "dataFinish",
    "posteriorStart": "posteriorStart", "posteriorFinish": "posteriorFinish",
    "acceptStart": "acceptStart", "acceptFinish": "acceptFinish",
}


class Notifier:
    def __init__(self):
        for attr, name in EVENTS.items():
            setattr(self, attr, name)
        self.monitors = []

    def initialize(self, application):
        return self

    def register(self, monitor):
        self.monitors.append(monitor)
        return self

    @property
    def eager(self):
        """True when a registered monitor times the phases inside a stage, which needs them
        launched one by one rather than replayed from captured graphs."""
        return any(getattr(m, "needs_eager_phases", False) for m in self.monitors)

    def notify(self, event, controller):
        for m in self.monitors:
            handler = getattr(m, event, None)
            if handler is not None:
                handler(controller=controller)
        return self


class CudaClock:
    """Marks on the current CUDA stream; durations resolved after a synchronisation."""

    def mark(self):
        import torch
        ev = torch.cuda.Event(enable_timing=True)
        ev.record(torch.cuda.current_stream())
        return ev

    def seconds(self, a, b):
        b.synchronize()
        return a.elapsed_time(b) / 1e3


class Profiler:
    """The reference's phase timers: the total time of every phase over the run."""

    PHASES = ("simulation", "samplePosterior", "prepareSamplingPDF", "beta", "walk", "chainAdvance", "verify",
              "prior", "data", "posterior", "accept", "resample")
    # phase -> (start event, finish event), Profiler.py:53-283
    SPANS = {"simulation": ("simulationStart", "simulationFinish"),
             "samplePosterior": ("samplePosteriorStart", "samplePosteriorFinish"),
             "prepareSamplingPDF": ("prepareSamplingPDFStart", "prepareSamplingPDFFinish"),
             "beta": ("betaStart", "betaFinish"), "walk": ("walkChainsStart", "walkChainsFinish"),
             "chainAdvance": ("chainAdvanceStart", "chainAdvanceFinish"),
             "verify": ("verifyStart", "verifyFinish"), "prior": ("priorStart", "priorFinish"),
             "data": ("dataStart", "dataFinish"), "posterior": ("posteriorStart", "posteriorFinish"),
             "accept": ("acceptStart", "acceptFinish"), "resample": ("resampleStart", "resampleFinish")}
    SEED = "prof-{wid:05}-{beta:03}x{parameters:03}x{chains:06}x{steps:03}.csv"
    needs_eager_phases = True

    def __init__(self, seed=SEED, directory=".", clock=None):
        self.seed = seed
        self.directory = directory
        self.clock = clock if clock is not None else CudaClock()
        self.beta = 0                              # β steps, as the reference's counter
        self.filename = None
        self._open = {}
        self._spans = {p: [] for p in self.PHASES}
        for phase, (start, finish) in self.SPANS.items():
            setattr(self, start, self._starter(phase))
            setattr(self, finish, self._finisher(phase, finish))

    def initialize(self, application):
        return self

    def _starter(self, phase):
        def handler(controller, **kwds):
            self._open[phase] = self.clock.mark()
        return handler

    def _finisher(self, phase, event):
        def handler(controller, **kwds):
            a = self._open.pop(phase, None)
            if a is not None:
                self._spans[phase].append((a, self.clock.mark()))
            if event == "betaFinish":
                self.beta += 1
            elif event == "simulationFinish":
                self.save(controller)
        return handler

    def totals(self):
        return {p: sum(self.clock.seconds(a, b) for a, b in self._spans[p]) for p in self.PHASES}

    def save(self, controller):
        """Write the timings in the reference's layout (Profiler.py:302-362)."""
        model = controller.model
        wid = getattr(controller.worker, "wid", 0)
        name = self.seed.format(wid=wid, beta=self.beta, parameters=model.parameters, chains=model.job.chains,
                                steps=model.job.steps)
        self.filename = os.path.join(self.directory, name)
        totals = self.totals()
        with open(self.filename, "w", newline="") as stream:
            w = csv.writer(stream)
            w.writerow(("run characteristics",))
            w.writerow(("beta steps", self.beta))
            w.writerow(("parameters", model.parameters))
            w.writerow(("chains", model.job.chains))
            w.writerow(("steps", model.job.steps))
            w.writerow(("timings",))
            for phase in self.PHASES:
                w.writerow((phase, totals[phase]))
        return self.filename
