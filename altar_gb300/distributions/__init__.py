"""Prior distributions (altar/altar/distributions)."""
from .uniform import Uniform

__all__ = ["Uniform"]
