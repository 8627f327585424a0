"""GB300 (sm_103a) implementation of AlTar's CATMIP hot path.

The reference's plugin surface (models, Annealer controller, Metropolis
sampler, COV scheduler, Grid solver) in Python over a C-ABI library of
hand-written CUDA kernels (``altar_gb300/csrc``); PyTorch provides device
buffers and streams only.
"""
from . import _native
from .application import Application

__all__ = ["Application", "_native"]
