"""Build and load the sm_103a C-ABI library ``libaltar_gb300.so``.

The library is compiled in-tree (``altar_gb300/_lib``) with nvcc for
``sm_103a`` only.  Loading is strict: there is no CPU fallback, so any use of
the GPU path without the built library raises :class:`NativeLibraryError`.
"""
import concurrent.futures
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBPATH = os.path.join(LIBDIR, "libaltar_gb300.so")
SOURCES = ("forward.cu", "stage.cu", "surrogate.cu", "linear.cu", "reverso.cu", "api.cu")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


class NativeLibraryError(RuntimeError):
    """The CUDA library is missing or failed to load."""


class AltarError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, name, code, message):
        super().__init__(f"{name} failed with status {code}: {message}")
        self.code = code


def _nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def build(verbose=False, force=False):
    """Compile csrc/*.cu for sm_103a (in parallel) and link the shared library."""
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "altar_gb300.h"))
    if (not force and os.path.exists(LIBPATH)
            and os.path.getmtime(LIBPATH) >= max(os.path.getmtime(d) for d in deps)):
        return LIBPATH
    nvcc = _nvcc()
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]
    # the FP32 forward models use explicit approximate reciprocals; flushing FP32
    # subnormals to zero lets them compile to the bare special-function instructions
    per_file = {"forward.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]}

    def compile_one(src):
        obj = os.path.join(LIBDIR, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *flags, *per_file.get(os.path.basename(src), []), "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise NativeLibraryError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose:
            print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise NativeLibraryError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIBPATH)
    return LIBPATH


# ---------------------------------------------------------------------------
# ctypes mirror of include/altar_gb300.h
c_int, c_int32, c_uint32, c_uint64 = ctypes.c_int, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64
c_size_t, c_double, c_void_p, c_char_p = ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p

AG_OK = 0
AG_MODEL_MOGI = 1
AG_MODEL_CDM = 2
AG_CHAIN_OUT_OF_SUPPORT = 1
AG_CHAIN_ABOVE_SURFACE = 2
AG_CHAIN_NONFINITE = 4
AG_DEV_ERR_TIMEOUT = 1
AG_DEV_ERR_NOT_SPD = 2
AG_STATION_TILE = 128


class StationSet(ctypes.Structure):
    _fields_ = [("xy", c_void_p), ("losd", c_void_p), ("weight", c_void_p), ("oid", c_void_p),
                ("m", c_int32), ("m_padded", c_int32), ("tile_box", c_void_p), ("order", c_void_p)]


class Layout(ctypes.Structure):
    _fields_ = [("nparams", c_int32), ("x_idx", c_int32), ("depth_idx", c_int32),
                ("strength_idx", c_int32), ("axes_idx", c_int32), ("omega_idx", c_int32),
                ("offset_idx", c_int32), ("log_strength", c_int32), ("nsources", c_int32),
                ("source_stride", c_int32), ("variant", c_int32), ("reserved", c_int32), ("nu", c_double)]


class LinearModel(ctypes.Structure):
    _fields_ = [("a64", c_void_p), ("b64", c_void_p), ("a_split", c_void_p), ("m_obs", c_int32), ("p", c_int32)]


class WhitenBlock(ctypes.Structure):
    _fields_ = [("w64", c_void_p), ("w_split", c_void_p), ("col0", c_int32), ("m", c_int32)]


class ReversoModel(ctypes.Structure):
    _fields_ = [("txy", c_void_p), ("d", c_void_p), ("w", c_void_p), ("n_obs", c_int32), ("nparams", c_int32),
                ("qin_idx", c_int32), ("hs_idx", c_int32), ("hd_idx", c_int32), ("as_idx", c_int32),
                ("ad_idx", c_int32), ("ac_idx", c_int32), ("east_cos", c_int32), ("reserved", c_int32),
                ("G", ctypes.c_double), ("v", ctypes.c_double), ("mu", ctypes.c_double),
                ("drho", ctypes.c_double), ("g", ctypes.c_double)]


class MLP(ctypes.Structure):
    _fields_ = [("nlayers", c_int32), ("sizes", c_int32 * 9)]


class StageState(ctypes.Structure):
    _fields_ = [("beta", c_void_p), ("dbeta_cov", c_void_p), ("scaling", c_void_p),
                ("sigma", c_void_p), ("chol", c_void_p), ("w", c_void_p),
                ("counters", c_void_p), ("epoch", c_void_p), ("dev_flags", c_void_p),
                ("chain0", c_int32), ("reserved", c_int32)]


P = c_void_p
_SIGNATURES = {
    "ag_last_error": (c_int, [c_char_p, c_size_t]),
    "ag_version": (c_char_p, []),
    "ag_forward_workspace_bytes": (c_size_t, [c_int, c_int32]),
    "ag_forward_variants": (c_int32, [c_int]),
    "ag_forward_llk": (c_int, [c_int, P, P, c_int32, P, c_double, P, P, P, P, P, c_size_t, P]),
    "ag_cdm_check": (c_int, [P, P, c_int32, P, P]),
    "ag_cdm_work": (c_int, [P, P, c_int32, P, P, P, P]),
    "ag_station_boxes": (c_int, [P, c_int32, c_int32, P, P]),
    "ag_forward_llk_subset": (c_int, [c_int, P, P, c_int32, P, c_double, P, P, P, P, P, P, c_size_t, P]),
    "ag_forward_llk_floor": (c_int, [c_int, P, P, c_int32, P, c_double, P, P, P, P, P, c_size_t, P]),
    "ag_forward_llk_subset_floor": (c_int, [c_int, P, P, c_int32, P, c_double, P, P, P, P, P, P, c_size_t, P]),
    "ag_da_floor": (c_int, [P, c_int32, c_uint64, c_uint32, P, P, P, P, P, P, P, P, P]),
    "ag_linear_kpad": (c_int32, [c_int32]),
    "ag_linear_prepare": (c_int, [P, c_int32, c_int32, P, P]),
    "ag_linear_workspace_bytes": (c_size_t, [c_int32, c_int32, c_int32]),
    "ag_linear_llk": (c_int, [P, P, c_int32, c_double, P, P, c_size_t, P, P]),
    "ag_linear_llk_fp64": (c_int, [P, P, c_int32, c_double, P, P]),
    "ag_whiten_workspace_bytes": (c_size_t, [c_int32, c_int32]),
    "ag_whiten_llk": (c_int, [P, P, c_int32, c_int32, P, P, c_size_t, P, P]),
    "ag_reverso_llk": (c_int, [P, P, c_int32, ctypes.c_double, P, P, P, P]),
    "ag_mlp_param_count": (ctypes.c_int64, [P]),
    "ag_mlp_activation_floats": (ctypes.c_int64, [P, c_int32]),
    "ag_normalize_inputs": (c_int, [P, c_int32, c_int32, P, P, P, P]),
    "ag_mlp_forward": (c_int, [P, P, P, P, c_int32, P, P, P]),
    "ag_mlp_backward": (c_int, [P, P, P, P, c_int32, P, P, P, P, P]),
    "ag_mse_grad": (c_int, [c_int32, c_int32, P, P, P, P, P]),
    "ag_adam_step": (c_int, [ctypes.c_int64, P, P, P, P, c_int32, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float, P, P]),
    "ag_to_bf16": (c_int, [ctypes.c_int64, P, P, P]),
    "ag_mlp_tc_pack_bytes": (c_size_t, [P]),
    "ag_mlp_tc_pack": (c_int, [P, P, P, P]),
    "ag_mlp_tc_workspace_bytes": (c_size_t, [P, c_int32]),
    "ag_mlp_forward_tc": (c_int, [P, P, P, P, c_int32, P, P, P, c_size_t, P, P]),
    "ag_surrogate_llk": (c_int, [c_int32, c_int32, P, P, P, P, c_double, c_double, P, P]),
    "ag_da_screen": (c_int, [P, c_int32, c_uint64, c_uint32, P, P, P, P, P, P, P, P, P]),
    "ag_da_moved": (c_int, [c_int32, c_int32, P, P, P, P, P, P]),
    "ag_da_accept": (c_int, [P, c_int32, c_int32, c_uint64, c_uint32, P, P, P, P, P, P, P, P, P, P, P,
                             P, P]),
    "ag_prior_sample": (c_int, [c_int32, c_int32, P, P, c_uint64, c_uint32, P, P, P]),
    "ag_prior_llk": (c_int, [P, c_int32, c_int32, P, P, P, P, P]),
    "ag_propose": (c_int, [P, P, c_int32, c_int32, P, P, c_uint64, c_uint32, P, P, P, P]),
    "ag_accept_floor": (c_int, [P, c_int32, c_uint64, c_uint32, P, P, P, P, P]),
    "ag_accept": (c_int, [P, c_int32, c_int32, c_uint64, c_uint32, P, P, P, P, P, P, P, P, P]),
    "ag_cov_workspace_bytes": (c_size_t, [c_int32]),
    "ag_cov_schedule": (c_int, [P, P, c_int32, c_double, c_double, P, c_size_t, P]),
    "ag_cov_schedule_brent": (c_int, [P, P, c_int32, c_double, c_double, c_int32, P, c_size_t, P]),
    "ag_cov_schedule_noalloc": (c_int, [P, P, c_int32, c_double, c_double, P]),
    "ag_cov_schedule_noalloc_max_chains": (c_int32, []),
    "ag_sigma_workspace_bytes": (c_size_t, [c_int32, c_int32]),
    "ag_weighted_cov": (c_int, [P, P, c_int32, c_int32, P, c_size_t, P]),
    "ag_cholesky_scaled": (c_int, [P, c_int32, P]),
    "ag_resample_workspace_bytes": (c_size_t, [c_int32]),
    "ag_resample": (c_int, [P, c_int32, c_int32, c_uint64, P, P, P, P, P, P, P, P, P, c_size_t, P]),
    "ag_adapt_scaling": (c_int, [P, c_double, c_double, P]),
    "ag_posterior": (c_int, [P, c_int32, P, P, P, P]),
    "ag_graph_begin": (c_int, [P]),
    "ag_graph_end": (c_int, [P, ctypes.POINTER(c_void_p)]),
    "ag_graph_launch": (c_int, [P, P]),
    "ag_graph_destroy": (c_int, [P]),
}

EXPORTED = tuple(_SIGNATURES)

_lib = None


def load(path=None):
    """Load the library (once) and declare the C signatures."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    path = path or LIBPATH
    if not os.path.exists(path):
        raise NativeLibraryError(
            f"{path} is missing: build it with altar_gb300._native.build() (nvcc, sm_103a)")
    try:
        lib = ctypes.CDLL(path)
    except OSError as e:
        raise NativeLibraryError(f"cannot load {path}: {e}") from e
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().ag_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def call(name, *args):
    """Call an ``int``-returning entry point and raise AltarError on failure."""
    rc = getattr(load(), name)(*args)
    if rc != AG_OK:
        raise AltarError(name, rc, last_error())
    return rc
