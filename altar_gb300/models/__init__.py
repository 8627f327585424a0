"""Model plugins (altar/altar/models, models/mogi, models/cdm)."""
from .bayesian import Bayesian
from .contiguous import Contiguous
from .cdm import CDM
from .mogi import Mogi
from .linear import Linear
from .densemogi import DenseMogi

__all__ = ["Bayesian", "Contiguous", "CDM", "Mogi", "Linear", "DenseMogi"]
