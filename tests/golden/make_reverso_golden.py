"""Generate the Reverso golden fixtures from the reference itself.

Run in a container that has the reference checkout (default path below, or
``--reference``); the GPU machines never run this script, they read the committed
``reverso_golden.npz``.

The reference's Python forward model ``models/reverso/reverso/libreverso.py:17-117``
(REVERSO, a generator of (u_r, u_z) per observation point; it needs only ``math``) is
imported directly and evaluated for seeded samples drawn from the priors of the
reference's example configuration (``models/reverso/examples/reverso.pfg``: Qin in
[0.4, 0.8], H_s in [2500, 3500], H_d in [3500, 4500], a_s, a_d, a_c in the ranges
below), at the observation points of its synthetic case (times 10^-6 .. 1 yr, 1-5 km
east; ``examples/synthetic/reverso.py``) plus seeded points scattered in ±6 km.
"""
import argparse
import importlib.util
import os

import numpy as np

YEAR = 365.25 * 24 * 3600
PRIORS = [(0.4, 0.8), (2500.0, 3500.0), (3500.0, 4500.0), (1500.0, 2500.0), (1500.0, 2500.0), (1.0, 2.0)]


def _load(root):
    path = os.path.join(root, "models", "reverso", "reverso", "libreverso.py")
    spec = importlib.util.spec_from_file_location("ref_libreverso", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "reverso_golden.npz"))
    args = ap.parse_args()
    lib = _load(args.reference)
    rng = np.random.default_rng(2024)
    synth = [(10.0 ** e * YEAR, float(r), 0.0) for e in range(-6, 1) for r in range(1000, 6000, 1000)]
    extra = [(float(t), float(x), float(y)) for t, x, y in zip(10.0 ** rng.uniform(-6, 0.5, 40) * YEAR,
                                                               rng.uniform(-6e3, 6e3, 40), rng.uniform(-6e3, 6e3, 40))]
    txy = np.array(synth + extra)
    theta = np.array([[rng.uniform(lo, hi) for lo, hi in PRIORS] for _ in range(16)])
    theta[0] = (0.6, 3.0e3, 4.0e3, 2.0e3, 2.2e3, 1.5)          # the synthetic case's truth
    material = dict(G=20.0e9, v=0.25, mu=2000.0, drho=300.0, g=9.81)
    ur = np.empty((len(theta), len(txy)))
    uz = np.empty_like(ur)
    for i, (Qin, H_s, H_d, a_s, a_d, a_c) in enumerate(theta):
        for j, (u_r, u_z) in enumerate(lib.REVERSO(locations=[tuple(p) for p in txy], H_s=H_s, H_d=H_d, a_s=a_s,
                                                   a_d=a_d, a_c=a_c, Qin=Qin, **material)):
            ur[i, j], uz[i, j] = u_r, u_z
    np.savez_compressed(args.out, theta=theta, txy=txy, u_r=ur, u_z=uz,
                        material=np.array([material[k] for k in ("G", "v", "mu", "drho", "g")]))
    print(f"wrote {args.out}: {len(theta)} samples x {len(txy)} points")


if __name__ == "__main__":
    main()
