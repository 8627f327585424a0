"""Random number source (replaces altar/altar/simulations/GSLRNG.py:25-53).

The reference draws from GSL's ranlxs2 seeded with ``seed``.  Here every draw
comes from the counter-based Philox4x32-10 generator keyed by ``seed`` and
addressed by (chain, stream, step, stage), so draws are reproducible and
independent of launch order; the streams are PRIOR (initial sample),
PROPOSAL (random-walk normals), ACCEPT (Metropolis dice) and RESAMPLE
(multinomial uniforms).
"""
from dataclasses import dataclass


@dataclass
class RNG:
    seed: int = 0
    algorithm: str = "philox4x32-10"

    def initialize(self, **kwds):
        self.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return self
