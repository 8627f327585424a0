"""CATMIP engine (altar/altar/bayesian): controller, sampler, scheduler, solvers."""
from .coolingstep import CoolingStep, StageState
from .notifier import Notifier, Profiler
from .metropolis import Metropolis
from .grid import Grid
from .brent import Brent
from .cov import COV
from .annealing import CUDAAnnealing
from .annealer import Annealer
from .sharding import ChainShards, ShardedAnnealing
from .surrogate import DelayedAcceptance, SubsetSurrogate, Surrogate

__all__ = ["CoolingStep", "StageState", "Notifier", "Profiler", "Metropolis", "Grid", "Brent", "COV",
           "CUDAAnnealing", "Annealer", "ChainShards", "ShardedAnnealing", "DelayedAcceptance", "Surrogate",
           "SubsetSurrogate"]
