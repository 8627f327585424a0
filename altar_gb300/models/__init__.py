"""Model plugins (altar/altar/models, models/mogi, models/cdm, models/linear, models/reverso)."""
from .bayesian import Bayesian
from .contiguous import Contiguous
from .cdm import CDM
from .mogi import Mogi
from .linear import Linear
from .densemogi import DenseMogi
from .reverso import Reverso

__all__ = ["Bayesian", "Contiguous", "CDM", "Mogi", "Linear", "DenseMogi", "Reverso"]
