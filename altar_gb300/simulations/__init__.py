"""Run configuration, random streams and output (altar/altar/simulations)."""
from .job import Job
from .rng import RNG
from .recorder import Recorder
from .checkpoint import Checkpoint

__all__ = ["Job", "RNG", "Recorder", "Checkpoint"]
