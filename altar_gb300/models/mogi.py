"""Mogi point source (models/mogi/mogi/Mogi.py, Source.py:39-73).

Parameter sets: ``location`` (2), ``depth`` (1), ``source`` (1 strength) and
optionally ``offsets``.  ``log_strength=True`` models log10 ΔV as the
reference does (mogi/Native.py:169); ``False`` models ΔV itself.  With
``sources=2`` the four sets hold two values each, source-major
([x1, y1, x2, y2], [d1, d2], [s1, s2]).
"""
from .. import _native
from .bayesian import Bayesian
from .forward import CUDA
from .observations import Observations


class Mogi(Bayesian):
    def __init__(self, psets, observations=None, case=None, nu=0.25, log_strength=True, sources=1,
                 autotune=False, **kwds):
        super().__init__(psets=psets, **kwds)
        self.autotune = bool(autotune)
        self.tuning = None
        self.nu = float(nu)
        self.log_strength = bool(log_strength)
        self.sources = int(sources)
        self.obs = observations if observations is not None else (
            Observations.read(case) if case is not None else None)
        self.strategy = None

    def initialize(self, application):
        super().initialize(application)
        if self.obs is None:
            raise ValueError("Mogi needs observations (arrays or a case directory)")
        self.initializeParameterSets()
        self.strategy = CUDA(_native.AG_MODEL_MOGI).initialize(application=application, model=self)
        return self

    @property
    def observations(self):
        return self.obs.observations

    def layout(self):
        p = self.psets
        off = p["offsets"].offset if "offsets" in p else -1
        if self.sources == 1:
            return _native.Layout(self.parameters, p["location"].offset, p["depth"].offset,
                                  p["source"].offset, -1, -1, off, int(self.log_strength), 1, 0, nu=self.nu)
        raise NotImplementedError("multi-source layouts are built with Mogi.layout_multi")

    def initializeSample(self, step, attempt=0, redraw=None):
        super().initializeSample(step, attempt=attempt, redraw=redraw)
        if self.autotune and redraw is None:
            from ..autotune import tune
            self.tuning = tune(self.strategy, step.theta)     # chains per CTA of the Mogi kernel
        return self

    def dataLikelihood(self, step):
        self.strategy.dataLikelihood(model=self, step=step)
        return self
