"""Build and call the C restatement ``oracle/csrc/catmip_ref.c`` (oracle; CPU baseline).

Test infrastructure only.  The library is compiled with plain gcc (portable
flags, no host-specific instructions) into ``oracle/_lib``.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc", "catmip_ref.c")
LIB = os.path.join(HERE, "_lib", "libcatmip_ref.so")


class RefLayout(ctypes.Structure):
    _fields_ = [("nparams", ctypes.c_int), ("x_idx", ctypes.c_int), ("depth_idx", ctypes.c_int),
                ("strength_idx", ctypes.c_int), ("axes_idx", ctypes.c_int),
                ("omega_idx", ctypes.c_int), ("log_strength", ctypes.c_int), ("nu", ctypes.c_double)]


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-pthread", "-std=c11", "-D_GNU_SOURCE", SRC, "-o",
           LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.ref_llk.restype = ctypes.c_int
        P = ctypes.c_void_p
        _lib.ref_llk.argtypes = [ctypes.c_int, P, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int,
                                 ctypes.c_double, P, P, ctypes.c_int]
        _lib.ref_cdm_los.restype = ctypes.c_int
        _lib.ref_cdm_los.argtypes = [P, P, P, P, P, ctypes.c_int, P]
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def llk(model, theta, layout, x, y, los, d, weight, norm, nthreads=1):
    """Data log-likelihood of each row of theta; model 1 = Mogi, 2 = CDM."""
    lib = load()
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    n = theta.shape[0]
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, los, d, weight)]
    out = np.empty(n)
    inv = np.zeros(n, dtype=np.int32)
    lib.ref_llk(model, _p(theta), n, ctypes.byref(layout), *(_p(a) for a in arrs), arrs[0].size,
                float(norm), _p(out), _p(inv), int(nthreads))
    return out, inv.astype(bool)


def cdm_los(theta_row, layout, x, y, los):
    lib = load()
    th = np.ascontiguousarray(theta_row, dtype=np.float64)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, los)]
    out = np.empty(arrs[0].size)
    bad = lib.ref_cdm_los(_p(th), ctypes.byref(layout), *(_p(a) for a in arrs), arrs[0].size, _p(out))
    return out, bool(bad)
