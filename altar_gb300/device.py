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


def hilbert_order(x, y, bits=16):
    """Permutation that sorts points along a Hilbert curve over their bounding square (the
    classic xy → d map, quadrant by quadrant): consecutive points of the result lie close
    together, so tiles of consecutive points have small bounding boxes."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = 1 << bits
    span = max(float(x.max() - x.min()), float(y.max() - y.min()), 1e-300)
    qx = ((x - x.min()) / span * (n - 1)).astype(np.int64)
    qy = ((y - y.min()) / span * (n - 1)).astype(np.int64)
    d = np.zeros_like(qx)
    s = n >> 1
    while s > 0:
        rx = ((qx & s) > 0).astype(np.int64)
        ry = ((qy & s) > 0).astype(np.int64)
        d += s * s * ((3 * rx) ^ ry)
        # rotate the quadrant so that the curve inside it starts and ends at its neighbours
        flip = (ry == 0) & (rx == 1)
        qx = np.where(flip, n - 1 - qx, qx)
        qy = np.where(flip, n - 1 - qy, qy)
        swap = ry == 0
        qx, qy = np.where(swap, qy, qx), np.where(swap, qx, qy)
        s >>= 1
    return np.argsort(d, kind="stable")


class Stations:
    """Observation points, LOS vectors, observed LOS displacements and weights.

    Device-resident counterpart of the state the reference attaches to its CUDA
    sources (libcudacdm.locations / los / data / oid, models/cdm/cdm/CUDA.py:25-68).
    ``weight`` is 1/σ² of each observation (diagonal data covariance).

    reorder: store the observations along a Hilbert curve (the CDM then picks its
    quadrature per tile of nearby stations).  The kernels' residual rows stay in the
    caller's order (``order``); ``data_rows`` and ``weight_rows`` are the observed values
    and weights in that order.
    """

    def __init__(self, x, y, los, d, weight, oid=None, reorder=False):
        x = np.asarray(x, dtype=np.float64)
        y = np.asarray(y, dtype=np.float64)
        m = x.size
        tile = _native.AG_STATION_TILE
        mp = ((m + tile - 1) // tile) * tile
        los = np.asarray(los, dtype=np.float64).reshape(m, 3)
        d = np.broadcast_to(np.asarray(d, dtype=np.float64), (m,))
        weight = np.broadcast_to(np.asarray(weight, dtype=np.float64), (m,))
        perm = hilbert_order(x, y) if reorder and m > 1 else np.arange(m)
        xy = np.zeros((mp, 4), dtype=np.float32)
        xy[:m, 0], xy[:m, 1] = split_hilo(x[perm])
        xy[:m, 2], xy[:m, 3] = split_hilo(y[perm])
        losd = np.zeros((mp, 4), dtype=np.float32)
        losd[:m, :3] = los[perm]
        losd[:m, 3] = d[perm]
        w = np.zeros(mp, dtype=np.float32)
        w[:m] = weight[perm]
        self.m, self.m_padded = m, mp
        self.xy = torch.from_numpy(xy).to(DEVICE)
        self.losd = torch.from_numpy(losd).to(DEVICE)
        self.weight = torch.from_numpy(w).to(DEVICE)
        rows_d = np.zeros(mp, dtype=np.float32)
        rows_d[:m] = d
        rows_w = np.zeros(mp, dtype=np.float32)
        rows_w[:m] = weight
        self.data_rows = torch.from_numpy(rows_d).to(DEVICE)
        self.weight_rows = torch.from_numpy(rows_w).to(DEVICE)
        if reorder:
            order = np.arange(mp, dtype=np.int32)
            order[:m] = perm
            self.order = torch.from_numpy(order).to(DEVICE)
        else:
            self.order = None
        if oid is not None:
            o = np.zeros(mp, dtype=np.int32)
            o[:m] = np.asarray(oid, dtype=np.int32)[perm]
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
                                          m, mp, self.tile_box.data_ptr(),
                                          self.order.data_ptr() if self.order is not None else None)

    @property
    def struct(self):
        return ctypes.byref(self._struct)
