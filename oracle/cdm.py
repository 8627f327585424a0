"""FP64 restatement of the Compound Dislocation Model surface displacements.

Oracle only (test infrastructure).  Follows the reference's numpy CDM
``models/cdm/cdm/libcdm.py`` (Nikkhoo et al. 2016), which is the only
reference implementation of the CDM that reproduces the Matlab goldens; the
reference C++ (``models/cdm/lib/libcdm/cdm.cc``) and CUDA
(``models/cdm/lib/libcudacdm/displacements.cu``) versions are not used as
oracles because they disagree with those goldens.

Units: station coordinates, centroid, depth and semi-axes in one length unit
(metres in the workloads), angles in degrees, opening in the length unit.
"""
import numpy as np


class AboveSurfaceError(ValueError):
    """The CDM reaches above the free surface (libcdm.py:222-224)."""


def rotation(omega_x, omega_y, omega_z):
    """R = Rz·Ry·Rx for clockwise rotations in degrees (libcdm.py:180-199)."""
    cx, sx = np.cos(np.radians(omega_x)), np.sin(np.radians(omega_x))
    cy, sy = np.cos(np.radians(omega_y)), np.sin(np.radians(omega_y))
    cz, sz = np.cos(np.radians(omega_z)), np.sin(np.radians(omega_z))
    rx = np.array([[1.0, 0.0, 0.0], [0.0, cx, sx], [0.0, -sx, cx]])
    ry = np.array([[cy, 0.0, -sy], [0.0, 1.0, 0.0], [sy, 0.0, cy]])
    rz = np.array([[cz, sz, 0.0], [-sz, cz, 0.0], [0.0, 0.0, 1.0]])
    return rz @ (ry @ rx)


def vertices(x0, y0, depth, ax, ay, az, omega_x, omega_y, omega_z):
    """The three rectangles' corners (libcdm.py:174-217).

    Returns a (3, 4, 3) array: rectangle k ∈ {P, Q, R} (normal to the body
    x, y, z axis respectively), corner 1..4, EFCS coordinate.
    """
    R = rotation(omega_x, omega_y, omega_z)
    ex, ey, ez = R[:, 0], R[:, 1], R[:, 2]
    lx, ly, lz = 2.0 * ax, 2.0 * ay, 2.0 * az          # full axes
    c = np.array([x0, y0, -depth], dtype=np.float64)
    p1 = c + 0.5 * ly * ey + 0.5 * lz * ez
    p2 = p1 - ly * ey
    p3 = p2 - lz * ez
    p4 = p1 - lz * ez
    q1 = c - 0.5 * lx * ex + 0.5 * lz * ez
    q2 = q1 + lx * ex
    q3 = q2 - lz * ez
    q4 = q1 - lz * ez
    r1 = c + 0.5 * lx * ex + 0.5 * ly * ey
    r2 = r1 - lx * ex
    r3 = r2 - ly * ey
    r4 = r1 - ly * ey
    return np.array([[p1, p2, p3, p4], [q1, q2, q3, q4], [r1, r2, r3, r4]])


def angular_dislocation(y1, y2, beta, b1, b2, b3, nu, a):
    """Surface displacement of one angular dislocation (libcdm.py:375-430).

    y1, y2: station coordinates in the angular-dislocation frame; beta: the
    dislocation angle; (b1, b2, b3): slip in that frame; a: depth of the
    dislocation vertex (positive down).
    """
    sb, cb = np.sin(beta), np.cos(beta)
    cot = 1.0 / np.tan(beta)
    k = 1.0 - 2.0 * nu
    z1 = y1 * cb + a * sb
    z3 = y1 * sb - a * cb
    r = np.sqrt(y1 * y1 + y2 * y2 + a * a)
    rpa = r + a
    rmz = r - z3
    fi = 2.0 * np.arctan2(y2, rpa / np.tan(0.5 * beta) - y1)
    lpa = np.log(rpa)
    lmz = np.log(rmz)
    s = 0.5 / np.pi
    v1 = b1 * s * ((1.0 - k * cot * cot) * fi
                   + y2 / rpa * (k * (cot + y1 / (2.0 * rpa)) - y1 / r)
                   - y2 * (r * sb - y1) * cb / (r * rmz))
    v2 = b1 * s * (k * ((0.5 + cot * cot) * lpa - cot / sb * lmz)
                   - (k * (y1 * cot - 0.5 * a - y2 * y2 / (2.0 * rpa)) + y2 * y2 / r) / rpa
                   + y2 * y2 * cb / (r * rmz))
    v3 = b1 * s * (k * fi * cot + y2 / rpa * (2.0 * nu + a / r)
                   - y2 * cb / rmz * (cb + a / r))
    v1 = v1 + b2 * s * (-k * ((0.5 - cot * cot) * lpa + cot * cot * cb * lmz)
                        - (k * (y1 * cot + 0.5 * a + y1 * y1 / (2.0 * rpa)) - y1 * y1 / r) / rpa
                        + z1 * (r * sb - y1) / (r * rmz))
    v2 = v2 + b2 * s * ((1.0 + k * cot * cot) * fi
                        - y2 / rpa * (k * (cot + y1 / (2.0 * rpa)) - y1 / r)
                        - y2 * z1 / (r * rmz))
    v3 = v3 + b2 * s * (-k * cot * (lpa - cb * lmz)
                        - y1 / rpa * (2.0 * nu + a / r)
                        + z1 / rmz * (cb + a / r))
    v1 = v1 + b3 * s * (y2 * (r * sb - y1) * sb / (r * rmz))
    v2 = v2 + b3 * s * (-y2 * y2 * sb / (r * rmz))
    v3 = v3 + b3 * s * (fi + y2 * (r * cb + a) * sb / (r * rmz))
    return v1, v2, v3


def side_pair(X, Y, bvec, pa, pb, nu):
    """Angular-dislocation pair on one side PA→PB of a rectangle (libcdm.py:310-372)."""
    side = pb - pa
    beta = np.arccos(-side[2] / np.sqrt(side @ side))
    eps = np.spacing(1.0)
    if abs(beta) < eps or abs(np.pi - beta) < eps:
        z = np.zeros(np.shape(X))
        return z, z.copy(), z.copy()
    e1 = np.array([side[0], side[1], 0.0])
    e1 /= np.sqrt(e1 @ e1)
    e2 = np.array([e1[1], -e1[0], 0.0])          # (-ez) × e1
    # EFCS -> ADCS: rows e1, e2, -ez
    y1a = e1[0] * (X - pa[0]) + e1[1] * (Y - pa[1])
    y2a = e2[0] * (X - pa[0]) + e2[1] * (Y - pa[1])
    y1ab = e1 @ side
    y2ab = e2 @ side
    y1b = y1a - y1ab
    y2b = y2a - y2ab
    b1 = e1 @ bvec
    b2 = e2 @ bvec
    b3 = -bvec[2]
    conf1 = (beta * y1a) >= 0                      # configuration I (libcdm.py:344)
    beff = np.where(conf1, beta - np.pi, beta)
    va = angular_dislocation(y1a, y2a, beff, b1, b2, b3, nu, -pa[2])
    vb = angular_dislocation(y1b, y2b, beff, b1, b2, b3, nu, -pb[2])
    v1, v2, v3 = vb[0] - va[0], vb[1] - va[1], vb[2] - va[2]
    # ADCS -> EFCS: columns e1, e2, -ez
    ue = e1[0] * v1 + e2[0] * v2
    un = e1[1] * v1 + e2[1] * v2
    uv = -v3
    return ue, un, uv


def rectangle(X, Y, corners, opening, nu):
    """Rectangular dislocation of tensile slip (libcdm.py:250-273)."""
    p1, p2, p3, p4 = corners
    n = np.cross(p2 - p1, p4 - p1)
    n = n / np.sqrt(n @ n)
    b = opening * n
    ue = np.zeros(np.shape(X))
    un = np.zeros(np.shape(X))
    uv = np.zeros(np.shape(X))
    for pa, pb in ((p1, p2), (p2, p3), (p3, p4), (p4, p1)):
        e, n_, v = side_pair(X, Y, b, pa, pb, nu)
        ue += e
        un += n_
        uv += v
    return ue, un, uv


def cdm(X, Y, x0, y0, depth, ax, ay, az, omega_x, omega_y, omega_z, opening, nu):
    """East, north and vertical surface displacements of a CDM (libcdm.py:39-247).

    Raises AboveSurfaceError when any corner lies above the free surface.
    """
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    v = vertices(x0, y0, depth, ax, ay, az, omega_x, omega_y, omega_z)
    if np.any(v[:, :, 2] > 0):
        raise AboveSurfaceError("the CDM must lie under the free surface")
    zero = np.zeros(np.shape(X))
    if ax == 0 and ay == 0 and az == 0:
        return zero, zero.copy(), zero.copy()
    if ax == 0 and ay != 0 and az != 0:
        return rectangle(X, Y, v[0], opening, nu)
    if ax != 0 and ay == 0 and az != 0:
        return rectangle(X, Y, v[1], opening, nu)
    if ax != 0 and ay != 0 and az == 0:
        return rectangle(X, Y, v[2], opening, nu)
    ue, un, uv = zero.copy(), zero.copy(), zero.copy()
    for k in range(3):
        e, n, w = rectangle(X, Y, v[k], opening, nu)
        ue += e
        un += n
        uv += w
    return ue, un, uv


def above_surface(x0, y0, depth, ax, ay, az, omega_x, omega_y, omega_z):
    """True where some corner of the CDM is above the surface (libcdm.py:219-224)."""
    v = vertices(x0, y0, depth, ax, ay, az, omega_x, omega_y, omega_z)
    return bool(np.any(v[:, :, 2] > 0))


def los_displacements(theta_row, layout, X, Y, los, nu):
    """Predicted LOS displacement of one sample (cdm/Source.py:48-91).

    theta_row: one sample; layout: dict with the indices x, y, depth,
    opening, ax, omega (as in CDM.py:235-245); los: (M, 3) unit vectors.
    """
    L = layout
    ue, un, uv = cdm(X, Y, theta_row[L["x"]], theta_row[L["x"] + 1], theta_row[L["depth"]],
                     theta_row[L["ax"]], theta_row[L["ax"] + 1], theta_row[L["ax"] + 2],
                     theta_row[L["omega"]], theta_row[L["omega"] + 1], theta_row[L["omega"] + 2],
                     theta_row[L["opening"]], nu)
    return ue * los[:, 0] + un * los[:, 1] + uv * los[:, 2]
