"""Data norms (altar/altar/norms)."""
from .l2 import L2

__all__ = ["L2"]
