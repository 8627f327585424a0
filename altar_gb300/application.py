"""Application shell (altar/altar/shells/Application.py:41-58), without pyre.

Holds the job, the random source, the controller and the model, and runs
model.initialize → controller.initialize → model.posterior.
"""
from .bayesian import Annealer
from .simulations import RNG, Job


class Application:
    def __init__(self, model, job=None, rng=None, controller=None, monitors=None):
        self.model = model
        self.job = job if job is not None else Job()
        self.rng = rng if rng is not None else RNG()
        self.controller = controller if controller is not None else Annealer()
        self.monitors = dict(monitors or {})

    def initialize(self):
        self.job.initialize(application=self)
        self.rng.initialize()
        self.model.initialize(application=self)
        self.controller.initialize(application=self)
        return self

    def run(self):
        self.initialize()
        return self.model.posterior(application=self)
