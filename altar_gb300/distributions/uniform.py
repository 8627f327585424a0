"""Uniform prior (altar/altar/distributions/Uniform.py:21-72, Base.py:44-79).

On the device the prior is applied to the whole sample at once: a model
collects the supports of its parameter sets into per-parameter bounds
(lo, hi) and the kernels draw the initial sample (gsl_ran_flat semantics,
a(1-u) + b u), verify the support (lo <= θ <= hi, closed as in
Uniform.verify) and add -log(hi - lo) per parameter to the prior
log-likelihood (log of the flat density, Base.priorLikelihood).
"""


class Uniform:
    def __init__(self, support=(0.0, 1.0)):
        lo, hi = (float(v) for v in support)
        if not hi > lo:
            raise ValueError(f"empty support {support}")
        self.support = (lo, hi)
        self.parameters = 0

    def initialize(self, rng=None):
        return self

    def bounds(self, count):
        lo, hi = self.support
        return [lo] * count, [hi] * count
