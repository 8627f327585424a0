"""Contiguous parameter set (altar/altar/models/Contiguous.py:19-127)."""
from ..distributions import Uniform


class Contiguous:
    def __init__(self, count=1, prior=None, prep=None):
        self.count = int(count)
        self.prior = prior if prior is not None else Uniform()
        self.prep = prep if prep is not None else self.prior
        self.offset = 0

    def initialize(self, model, offset):
        """Record my offset in the sample vector and return my parameter count."""
        self.offset = offset
        self.prep.parameters = self.prior.parameters = self.count
        if not isinstance(self.prior, Uniform) or not isinstance(self.prep, Uniform):
            raise NotImplementedError("the device prior supports Uniform distributions only")
        return self.count

    def prior_bounds(self):
        return self.prior.bounds(self.count)

    def prep_bounds(self):
        return self.prep.bounds(self.count)
