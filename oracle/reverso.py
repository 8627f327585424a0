"""Reverso two-reservoir model: FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may use this module,
and only as the checker.

Restates the reference's forward model and data log-likelihood:
  * reverso: models/reverso/lib/libreverso/reverso.cc:37-105 (the C++ the default
    "fast" strategy calls through Source.cc:56-88), with its helper H at
    reverso.cc:109-142; the same algebra as the Python generator
    models/reverso/reverso/libreverso.py:17-117;
  * the two strategies' E/N convention: the C++ sets u_E = u_r cos φ, u_N = u_r sin φ
    (reverso.cc:92-96); the Python "analytic" strategy sets u_E = u_r sin φ,
    u_N = u_r cos φ (Native.py:96-100), as does the synthetic generator
    (examples/synthetic/reverso.py);
  * residuals r = u - d (Source.cc:92-123) and llk = norm - |L r|²/2 with
    L = chol(Cd⁻¹) (Fast.py:52-90, altar/altar/norms/L2.py:39-52), for the diagonal
    Cd the model builds from the σ² columns of displacements.csv (Reverso.py:94-106);
  * norm = -1/2 (log(2π)·n_points + log det Cd) with n_points the number of
    observation records, not of data values (Reverso.py:292-305).

The reference keeps its quirks and so does this restatement: the time constant uses
H_c ** γ_s (reverso.cc:60-61) and the pressures 1 - exp(-t/τ) (reverso.cc:79).
"""
import math

import numpy as np

PARAMS = ("Qin", "H_s", "H_d", "a_s", "a_d", "a_c")


def radial_vertical(th, txy, G=20.0e9, v=0.25, mu=2000.0, drho=300.0, g=9.81):
    """(u_r, u_z) at the observation points, as REVERSO yields them (libreverso.py:17-91).
    th: Qin, H_s, H_d, a_s, a_d, a_c (shape (6,), or (n, 6) for n samples at once, giving
    (n, n_points) arrays); txy: (n_points, 3) time (s), east, north (m)."""
    th = np.asarray(th, dtype=np.float64)
    Qin, H_s, H_d, a_s, a_d, a_c = (th[..., i, None] if th.ndim == 2 else float(th[i]) for i in range(6))
    pi = math.pi
    dPs0 = dPd0 = 0.0
    k = (a_d / a_s) ** 3
    H_c = H_d - H_s
    gamma_s = 8.0 * (1 - v) / (3.0 * pi)
    gamma_d = 8.0 * (1 - v) / (3.0 * pi)
    gamma_r = gamma_s + gamma_d * k
    tau = (8.0 * mu * H_c ** gamma_s * gamma_d * k * a_s ** 3) / (G * a_c ** 4 * gamma_r)
    A = gamma_d * k / gamma_r
    A *= dPd0 - dPs0 + drho * g * H_c - 8 * gamma_s * mu * Qin * H_c / (pi * a_c ** 4 * gamma_r)
    t, x, y = (np.asarray(txy, dtype=np.float64)[:, i] for i in range(3))
    f0 = A * (1.0 - np.exp(-t / tau))
    f1 = G * Qin * t / (pi * a_s ** 3 * gamma_r)
    dP_s = dPs0 + f1 + f0
    dP_d = dPd0 + f1 - f0 * gamma_s / (gamma_d * k)
    r2 = x * x + y * y
    r = np.sqrt(r2)
    H2_s, H2_d = H_s ** 2, H_d ** 2
    R2_s, R2_d = r2 + H2_s, r2 + H2_d
    alpha_s = 1.0 if gamma_s == 1.0 else 4.0 * H2_s / (pi * R2_s)
    alpha_d = 1.0 if gamma_d == 1.0 else 4.0 * H2_d / (pi * R2_d)
    f_s = a_s ** 3 * alpha_s * (1 - v) / (G * (H2_s + r2) ** 1.5)
    f_d = a_d ** 3 * alpha_d * (1 - v) / (G * (H2_d + r2) ** 1.5)
    u_r = r * f_s * dP_s + r * f_d * dP_d
    u_z = H_s * f_s * dP_s + H_d * f_d * dP_d
    return u_r, u_z


def displacements(th, txy, east_cos=True, **material):
    """(n_points, 3) displacements east, north, up of one sample (reverso.cc:92-100 when
    east_cos, else the convention of Native.py:96-100)."""
    u_r, u_z = radial_vertical(th, txy, **material)
    txy = np.asarray(txy, dtype=np.float64)
    phi = np.arctan2(txy[:, 2], txy[:, 1])
    c, s = np.cos(phi), np.sin(phi)
    if east_cos:
        return np.stack([u_r * c, u_r * s, u_z], 1)
    return np.stack([u_r * s, u_r * c, u_z], 1)


def normalization(var):
    """-1/2 (log(2π)·n_points + log det Cd) for the (n_points, 3) σ² of a diagonal Cd."""
    var = np.asarray(var, dtype=np.float64)
    return -0.5 * (math.log(2.0 * math.pi) * var.shape[0] + float(np.sum(np.log(var))))


def data_llk(theta, txy, d, var, norm=None, east_cos=True, **material):
    """Data log-likelihood of each row of theta (n, 6 in PARAMS order)."""
    norm = normalization(var) if norm is None else norm
    w = 1.0 / np.asarray(var, dtype=np.float64)
    u_r, u_z = radial_vertical(np.atleast_2d(theta), txy, **material)
    txy = np.asarray(txy, dtype=np.float64)
    phi = np.arctan2(txy[:, 2], txy[:, 1])
    c, s = np.cos(phi), np.sin(phi)
    ue, un = (u_r * c, u_r * s) if east_cos else (u_r * s, u_r * c)
    r2 = w[:, 0] * (ue - d[:, 0]) ** 2 + w[:, 1] * (un - d[:, 1]) ** 2 + w[:, 2] * (u_z - d[:, 2]) ** 2
    return norm - 0.5 * r2.sum(1)


def synthetic_points(year=365.25 * 24 * 3600):
    """Observation times and places of the reference's synthetic case
    (examples/synthetic/reverso.py makeTicks): t = 10^e yr for e = -6..0, r = 1..5 km
    along the east axis."""
    return np.array([(10.0 ** e * year, float(r), 0.0) for e in range(-6, 1) for r in range(1000, 6000, 1000)])


def synthetic_case(truth=(0.6, 3.0e3, 4.0e3, 2.0e3, 2.2e3, 1.5), **kw):
    """Displacements and σ² of the reference's synthetic case generator (noise-free data,
    σ² = max(0.05 u, 0.01)² per component as in examples/synthetic/reverso.py, with the
    generator's own E = u_r sin φ, N = u_r cos φ)."""
    txy = synthetic_points()
    u = displacements(truth, txy, east_cos=False, **kw)
    var = np.maximum(0.05 * u, 0.01) ** 2
    return txy, u, var
