"""The C ABI library: exported symbols and struct layouts (CPU, no GPU calls)."""
import ctypes
import os
import re
import subprocess

from altar_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "altar_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ag_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(native_lib):
    names = declared()
    assert len(names) >= 20
    for name in names:
        assert hasattr(native_lib, name), f"{name} declared in the header but not exported"
    assert set(names) <= set(_native.EXPORTED) | set(names)
    assert set(_native.EXPORTED) <= set(names), "Python binds a symbol the header does not declare"


def test_version_string(native_lib):
    assert b"sm_103a" in native_lib.ag_version()


def test_struct_layouts_match_header(tmp_path):
    src = tmp_path / "probe.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "altar_gb300.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu\\n\", sizeof(ag_station_set),"
        " sizeof(ag_layout), sizeof(ag_stage_state), offsetof(ag_layout, nu),"
        " offsetof(ag_station_set, m), offsetof(ag_stage_state, dev_flags)); printf(\"%zu\\n\", offsetof(ag_stage_state, chain0));"
        " printf(\"%zu %zu %zu\\n\", sizeof(ag_reverso_model), offsetof(ag_reverso_model, east_cos),"
        " offsetof(ag_reverso_model, G)); return 0;}\n")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(_native.StationSet), ctypes.sizeof(_native.Layout),
            ctypes.sizeof(_native.StageState), _native.Layout.nu.offset, _native.StationSet.m.offset,
            _native.StageState.dev_flags.offset, _native.StageState.chain0.offset, ctypes.sizeof(_native.ReversoModel),
            _native.ReversoModel.east_cos.offset, _native.ReversoModel.G.offset]
    assert got == want


def test_argument_errors_without_gpu(native_lib):
    """Host-side validation rejects bad arguments before touching the device."""
    rc = native_lib.ag_forward_llk(_native.AG_MODEL_CDM, None, None, 0, None, 0.0, None, None, None,
                                   None, None, 0, None)
    assert rc == 1
    assert "null" in _native.last_error().lower() or "invalid" in _native.last_error().lower()
    assert native_lib.ag_forward_workspace_bytes(_native.AG_MODEL_CDM, 10) > 0
    assert native_lib.ag_cov_workspace_bytes(0) == 0
    # the surrogate likelihood stages the k x k Gram matrix in shared memory: k <= 96
    p = ctypes.c_void_p(16)
    assert _native.load().ag_surrogate_llk(10, 97, p, p, p, p, 0.0, 0.0, p, None) == 1
    assert "96" in _native.last_error()
    # Reverso: parameter positions must lie inside the sample row
    m = _native.ReversoModel(16, 16, 16, 35, 6, 0, 1, 2, 3, 4, 6, 1, 0, 20e9, 0.25, 2000.0, 300.0, 9.81)
    assert _native.load().ag_reverso_llk(ctypes.byref(m), p, 4, 0.0, None, p, None, None) == 1
    assert "out of range" in _native.last_error()
