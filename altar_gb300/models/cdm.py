"""Compound Dislocation Model (models/cdm/cdm/CDM.py:21-457).

Parameter sets: ``location`` (2), ``depth`` (1), ``opening`` (1), ``a`` (3
semi-axes), ``omega`` (3 rotations, degrees), and optionally ``offsets`` (one
per dataset), as CDM.initializeParameterSets (CDM.py:218-248) — except that
``offsets`` may be absent.  Samples whose CDM reaches above the free surface
are rejected like out-of-support samples (the reference raises and aborts,
libcdm.py:222-224); the initial sample is redrawn until every chain is valid.
"""
import ctypes

import torch

from .. import _native
from ..device import DEVICE, ptr, stream_handle
from .bayesian import Bayesian
from .forward import CUDA
from .observations import Observations


class CDM(Bayesian):
    def __init__(self, psets, observations=None, case=None, nu=0.25, variant=0, autotune=False, **kwds):
        super().__init__(psets=psets, **kwds)
        self.nu = float(nu)
        self.variant = int(variant)
        self.autotune = bool(autotune)
        self.tuning = None
        self.obs = observations if observations is not None else (
            Observations.read(case) if case is not None else None)
        self.strategy = None

    def initialize(self, application):
        super().initialize(application)
        if self.obs is None:
            raise ValueError("CDM needs observations (arrays or a case directory)")
        self.initializeParameterSets()
        self.strategy = CUDA(_native.AG_MODEL_CDM).initialize(application=application, model=self)
        return self

    @property
    def observations(self):
        return self.obs.observations

    def layout(self):
        p = self.psets
        off = p["offsets"].offset if "offsets" in p else -1
        return _native.Layout(self.parameters, p["location"].offset, p["depth"].offset,
                              p["opening"].offset, p["a"].offset, p["omega"].offset, off, 0, 1, 0,
                              variant=self.variant, nu=self.nu)

    def initializeSample(self, step, max_attempts=1000):
        super().initializeSample(step)
        status = torch.zeros(step.samples, dtype=torch.int32, device=DEVICE)
        lay = self.layout()
        for attempt in range(1, max_attempts + 1):
            status.zero_()
            _native.call("ag_cdm_check", ctypes.byref(lay), ptr(step.theta), step.samples,
                         ptr(status), stream_handle())
            if int(torch.count_nonzero(status)) == 0:
                if self.autotune:
                    from ..autotune import tune
                    self.tuning = tune(self.strategy, step.theta)
                    self.variant = self.tuning["variant"]
                return self
            super().initializeSample(step, attempt=attempt, redraw=status)
        raise RuntimeError("could not draw an initial sample with every CDM below the surface")

    def dataLikelihood(self, step):
        self.strategy.dataLikelihood(model=self, step=step)
        return self

    def verify(self, step, mask):
        super().verify(step, mask)
        _native.call("ag_cdm_check", ctypes.byref(self.layout()), ptr(step.theta), step.samples,
                     ptr(mask), stream_handle())
        return mask
