"""Device buffers and argument marshalling for the C ABI.

PyTorch is used only as a CUDA allocator and stream provider: tensors hold
the device arrays, and their raw pointers are handed to the library.
"""
import ctypes

import numpy as np
import torch

from . import _native

DEVICE = torch.device("cuda")


def require_cuda():
    if not torch.cuda.is_available():
        raise _native.NativeLibraryError("a CUDA device is required: the GB300 path has no CPU fallback")
    _native.load()


def ptr(t):
    """Raw device pointer of a tensor (None stays NULL)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def workspace(nbytes):
    """A 256-byte aligned device workspace (torch allocations are 512-byte aligned)."""
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=DEVICE)


def split_hilo(v):
    """FP64 values as float32 pairs (hi + lo) that keep ~48 bits of the coordinate."""
    v = np.asarray(v, dtype=np.float64)
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


class Stations:
    """Observation points, LOS vectors, observed LOS displacements and weights.

    Device-resident counterpart of the state the reference attaches to its CUDA
    sources (libcudacdm.locations / los / data / oid, models/cdm/cdm/CUDA.py:25-68).
    ``weight`` is 1/σ² of each observation (diagonal data covariance).
    """

    def __init__(self, x, y, los, d, weight, oid=None):
        x = np.asarray(x, dtype=np.float64)
        m = x.size
        tile = _native.AG_STATION_TILE
        mp = ((m + tile - 1) // tile) * tile
        xy = np.zeros((mp, 4), dtype=np.float32)
        xy[:m, 0], xy[:m, 1] = split_hilo(x)
        xy[:m, 2], xy[:m, 3] = split_hilo(y)
        losd = np.zeros((mp, 4), dtype=np.float32)
        losd[:m, :3] = np.asarray(los, dtype=np.float64).reshape(m, 3)
        losd[:m, 3] = np.asarray(d, dtype=np.float64)
        w = np.zeros(mp, dtype=np.float32)
        w[:m] = np.asarray(weight, dtype=np.float64)
        self.m, self.m_padded = m, mp
        self.xy = torch.from_numpy(xy).to(DEVICE)
        self.losd = torch.from_numpy(losd).to(DEVICE)
        self.weight = torch.from_numpy(w).to(DEVICE)
        if oid is not None:
            o = np.zeros(mp, dtype=np.int32)
            o[:m] = np.asarray(oid, dtype=np.int32)
            self.oid = torch.from_numpy(o).to(DEVICE)
        else:
            self.oid = None
        # bounding box of each tile of stations (the CDM picks its quadrature per tile)
        self.tile_box = torch.empty(mp // tile, 4, dtype=torch.float32, device=DEVICE)
        _native.call("ag_station_boxes", ctypes.c_void_p(self.xy.data_ptr()), m, mp,
                     ctypes.c_void_p(self.tile_box.data_ptr()), stream_handle())
        self._struct = _native.StationSet(self.xy.data_ptr(), self.losd.data_ptr(),
                                          self.weight.data_ptr(),
                                          self.oid.data_ptr() if self.oid is not None else None,
                                          m, mp, self.tile_box.data_ptr())

    @property
    def struct(self):
        return ctypes.byref(self._struct)
