"""Generate the CDM golden fixtures from the reference itself.

Run in a container that has the reference checkout (default path below, or
``--reference``); the GPU machines never run this script, they read the
committed ``cdm_golden.npz``.

Two kinds of vectors are written:
  * ``matlab_*``: the 12-station Matlab golden test of the reference,
    ``models/cdm/tests/libcdm.py:27-46`` (inputs at ``:103-117``), parsed
    from that file as text;
  * ``ref_*``: outputs of the reference's numpy CDM,
    ``models/cdm/cdm/libcdm.py:39-247``, imported directly, for seeded
    random sources drawn from the CDM workload priors (centroid ±10 km,
    depth 1-10 km, rotations ±90°, semi-axes 0.1-3 km, opening ±50 m,
    ν = 0.25) on a 33-point grid over ±20 km plus a few near-field points.
"""
import argparse
import ast
import importlib.util
import os

import numpy as np


def _load_libcdm(root):
    path = os.path.join(root, "models", "cdm", "cdm", "libcdm.py")
    spec = importlib.util.spec_from_file_location("ref_libcdm", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _matlab_vectors(root):
    path = os.path.join(root, "models", "cdm", "tests", "libcdm.py")
    tree = ast.parse(open(path).read())
    arrays = {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            name = getattr(node.targets[0], "id", None)
            if name in ("X", "Y", "mde", "mdn", "mdv"):
                call = node.value
                arrays[name] = np.array(ast.literal_eval(call.args[0]), dtype=np.float64)
    return arrays


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "cdm_golden.npz"))
    args = ap.parse_args()

    lib = _load_libcdm(args.reference)
    mat = _matlab_vectors(args.reference)
    # the Matlab test source (models/cdm/tests/libcdm.py:103-117)
    matlab_src = np.array([0.5, -0.25, 2.75, 0.4, 0.45, 0.8, 5.0, -8.0, 30.0, 1e-3, 0.25])

    rng = np.random.default_rng(20240611)
    g = np.linspace(-20e3, 20e3, 33)
    GX, GY = np.meshgrid(g, g)
    X = np.concatenate([GX.ravel(), rng.uniform(-3e3, 3e3, 16)])
    Y = np.concatenate([GY.ravel(), rng.uniform(-3e3, 3e3, 16)])
    srcs, outs = [], []
    while len(srcs) < 24:
        x0, y0 = rng.uniform(-1e4, 1e4, 2)
        depth = rng.uniform(1e3, 1e4)
        om = rng.uniform(-90, 90, 3)
        a = rng.uniform(100, 3000, 3)
        op = rng.uniform(-50, 50)
        try:
            ue, un, uv = lib.CDM(X, Y, x0, y0, depth, a[0], a[1], a[2], om[0], om[1], om[2], op, 0.25)
        except ValueError:
            continue                              # above the free surface: not a valid source
        srcs.append([x0, y0, depth, a[0], a[1], a[2], om[0], om[1], om[2], op, 0.25])
        outs.append(np.stack([ue, un, uv]))
    # also record the reference's outputs at the Matlab points
    ue, un, uv = lib.CDM(mat["X"], mat["Y"], *matlab_src)
    np.savez_compressed(
        args.out,
        matlab_X=mat["X"], matlab_Y=mat["Y"],
        matlab_ue=mat["mde"], matlab_un=mat["mdn"], matlab_uv=mat["mdv"],
        matlab_src=matlab_src,
        matlab_ref=np.stack([ue, un, uv]),
        ref_X=X, ref_Y=Y, ref_src=np.array(srcs), ref_u=np.array(outs),
    )
    print("wrote", args.out, len(srcs), "sources x", X.size, "stations")


if __name__ == "__main__":
    main()
