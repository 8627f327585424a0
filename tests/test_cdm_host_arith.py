"""The CDM likelihood kernel's arithmetic, compiled for the host (no GPU).

tests/cdm_host/cdm_host.cpp builds altar_gb300/csrc/cdm_side.cuh with g++, the device
intrinsics replaced by correctly rounded host operations.  Checked here:
  * the formulas against the FP64 oracle (models/cdm/cdm/libcdm.py restated in
    oracle/cdm.py) on prior sources: rectangles near the free surface by their
    angular-dislocation pairs, the others by quadrature of point tensile dislocations;
    one normwise tolerance for every source, near-vertical sides included;
  * the per-chain plan (which rectangles are integrated, with how many nodes);
  * the static FP32 operation counts of one pair and one quadrature node against the
    library's constants, which ag_cdm_work (the bench's roofline) sums per chain;
  * the Gauss-Legendre table against an independent computation.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import cdm

from gpu_helpers import CDM_LAYOUT, LOS, cdm_prior_rows, min_vertical_angle

HERE = os.path.dirname(os.path.abspath(__file__))
P = ctypes.POINTER


@pytest.fixture(scope="module")
def host(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    so = str(tmp_path_factory.mktemp("cdm_host") / "cdm_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                    os.path.join(HERE, "cdm_host", "cdm_host.cpp"), "-o", so], check=True)
    lib = ctypes.CDLL(so)
    lib.cdm_host_los.argtypes = [P(ctypes.c_double), ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double),
                                 P(ctypes.c_double), ctypes.c_double, P(ctypes.c_double)]
    lib.cdm_host_los.restype = ctypes.c_int
    lib.cdm_host_side_counts.argtypes = [P(ctypes.c_long)] * 4
    lib.cdm_host_quad_counts.argtypes = [P(ctypes.c_long)] * 4
    lib.cdm_host_work_constants.argtypes = [P(ctypes.c_int)]
    lib.cdm_host_plan.argtypes = [P(ctypes.c_double), ctypes.c_double, P(ctypes.c_float), ctypes.c_int,
                                  P(ctypes.c_uint32), P(ctypes.c_int), P(ctypes.c_double), P(ctypes.c_double)]
    return lib


def _dp(a):
    return a.ctypes.data_as(P(ctypes.c_double))


def _constants(host):
    k = (ctypes.c_int * 8)()
    host.cdm_host_work_constants(k)
    return dict(zip(["side", "steep_extra", "quad_rect", "quad_node", "station", "sfu_side", "sfu_steep_extra",
                     "sfu_quad_node"], list(k)))


def test_flop_counts_match_library_constants(host):
    """Counted by evaluating a pair and a quadrature rectangle with a counting number type
    (FMA = 2); the library's work count (ag_cdm_work) uses the constants."""
    k = _constants(host)
    flop, sfu, flop_s, sfu_s = (ctypes.c_long() for _ in range(4))
    host.cdm_host_side_counts(ctypes.byref(flop), ctypes.byref(sfu), ctypes.byref(flop_s), ctypes.byref(sfu_s))
    assert (flop.value, sfu.value) == (k["side"], k["sfu_side"])
    assert (flop_s.value - flop.value, sfu_s.value - sfu.value) == (k["steep_extra"], k["sfu_steep_extra"])
    f1, s1, f2, s2 = (ctypes.c_long() for _ in range(4))
    host.cdm_host_quad_counts(ctypes.byref(f1), ctypes.byref(s1), ctypes.byref(f2), ctypes.byref(s2))
    assert f2.value - f1.value == k["quad_node"] and s2.value - s1.value == k["sfu_quad_node"]
    assert f1.value - k["quad_node"] == k["quad_rect"] and s1.value == k["sfu_quad_node"]
    # per station besides the rectangles: relative coordinates (6), LOS projection (5),
    # residual (1), float-float w·r² accumulation (19)
    assert k["station"] == 31


def _plan(host, th, box=None, m=1):
    """Plan of one source and the work over m stations in tiles with the given boxes (default:
    one station at the source centre, the tile closest to every rectangle)."""
    mask, f, u = ctypes.c_uint32(), ctypes.c_double(), ctypes.c_double()
    nq = (ctypes.c_int * 6)()
    t = np.ascontiguousarray(th, dtype=np.float64)
    if box is None:
        box = np.array([[th[0], th[0], th[1], th[1]]], dtype=np.float32)
    box = np.ascontiguousarray(box, dtype=np.float32)
    assert host.cdm_host_plan(_dp(t), 0.25, box.ctypes.data_as(P(ctypes.c_float)), m, ctypes.byref(mask), nq,
                              ctypes.byref(f), ctypes.byref(u)) == 0
    return mask.value, np.array(list(nq)).reshape(3, 2), f.value


def _thresholds():
    import re
    text = open(os.path.join(HERE, "..", "altar_gb300", "csrc", "cdm_side.cuh")).read()
    body = re.search(r"kQuadDelta2\[kGaussMax\] = \{([^}]*)\}", text).group(1)
    return np.array([float(v.strip().rstrip("f")) for v in body.replace("\n", " ").split(",") if v.strip()],
                    dtype=np.float32)


def _nodes(delta2):
    """Smallest n with δ² >= δ_n² (17 if none), as the library's threshold search."""
    T = _thresholds().astype(np.float64)
    for n in range(1, 17):
        if delta2 >= T[n - 1]:
            return n
    return 17


def test_quadrature_thresholds():
    """δ_n² is the smallest δ² at which n nodes per direction meet ρ^(-2n) <= 1e-7
    (ρ = δ + sqrt(δ² + 1)), rounded up to FP32: n - 1 nodes do not meet it there."""
    T = _thresholds().astype(np.float64)
    for n in range(1, 17):
        d = np.sqrt(T[n - 1])
        rho = d + np.sqrt(d * d + 1)
        assert rho ** (-2 * n) <= 1e-7 * (1 + 1e-6)
        if n > 1:
            assert rho ** (-2 * (n - 1)) > 1e-7
        rho_n = 1e-7 ** (-1.0 / (2 * n))
        exact = ((rho_n - 1 / rho_n) / 2) ** 2
        assert exact <= T[n - 1] <= exact * (1 + 2 ** -22)


def test_plan_quadrature_far_rectangles(host):
    """A rectangle is integrated everywhere ("far") with n1 x n2 nodes, n_i the smallest n
    with ρ_i^(-2n) <= 1e-7 (ρ = δ + sqrt(δ² + 1), δ = depth of the shallowest corner / half
    side), when n1 n2 <= 32; otherwise its sides are evaluated (over the tiles where they
    cost less than the quadrature: here a tile at the source, the same as the chain plan)."""
    from oracle import cdm as ocdm
    k = _constants(host)
    nquad = 0
    for th in cdm_prior_rows(200, seed=21):
        mask, nq, flop = _plan(host, th)
        V = ocdm.vertices(th[0], th[1], th[2], *th[4:7], *th[7:10])
        work = k["station"]
        for r in range(3):
            h1 = np.linalg.norm(V[r][1] - V[r][0]) / 2
            h2 = np.linalg.norm(V[r][3] - V[r][0]) / 2
            D = -V[r][:, 2].max()
            n = [_nodes((D * D) / (h * h)) for h in (h1, h2)]
            quad = max(n) <= 16 and n[0] * n[1] <= 32
            assert bool(mask >> (24 + r) & 1) == quad
            sides = (mask >> (4 * r)) & 0xF
            if quad:
                assert list(nq[r]) == n and sides == 0
                work += k["quad_rect"] + k["quad_node"] * n[0] * n[1]
                nquad += 1
            else:
                steep = (mask >> (12 + 4 * r)) & 0xF
                work += bin(sides).count("1") * k["side"] + bin(steep).count("1") * k["steep_extra"]
        assert flop == work
    assert 0.3 < nquad / 600 < 0.9


def test_gauss_legendre_table():
    """The nodes and weights of altar_gb300/csrc/gauss_legendre.cuh against numpy's rules."""
    import re
    text = open(os.path.join(HERE, "..", "altar_gb300", "csrc", "gauss_legendre.cuh")).read()
    tables = {}
    for name in ("kGaussX", "kGaussW"):
        body = re.search(name + r"\[\d+\] = \{([^}]*)\}", text).group(1)
        tables[name] = np.array([float(v) for v in body.replace("\n", " ").split(",") if v.strip()])
    for n in range(1, 17):
        x, w = np.polynomial.legendre.leggauss(n)
        o = n * (n - 1) // 2
        np.testing.assert_allclose(tables["kGaussX"][o:o + n], x, rtol=0, atol=1e-15)
        np.testing.assert_allclose(tables["kGaussW"][o:o + n], w, rtol=1e-14)


def test_side_arithmetic_against_oracle(host):
    g = np.linspace(-20e3, 20e3, 30)
    X, Y = [np.ascontiguousarray(a.ravel()) for a in np.meshgrid(g, g)]
    los = np.ascontiguousarray(np.tile(LOS, (X.size, 1)))
    theta = cdm_prior_rows(24, seed=3)
    errs, flat = [], []
    for th in theta:
        ref = cdm.los_displacements(th, CDM_LAYOUT, X, Y, los, 0.25)
        out = np.empty(X.size)
        t = np.ascontiguousarray(th, dtype=np.float64)
        assert host.cdm_host_los(_dp(t), X.size, _dp(X), _dp(Y), _dp(los), 0.25, _dp(out)) == 0
        errs.append(np.max(np.abs(out - ref)) / np.max(np.abs(ref)))
        flat.append(min_vertical_angle(th) >= 10.0)
    errs, flat = np.array(errs), np.array(flat)
    assert flat.sum() >= 16
    # one tolerance whatever the angle of the sides (near-vertical sides included)
    assert np.all(errs <= 5e-6), errs.max()
    assert np.median(errs) <= 1e-6, np.median(errs)


def test_steep_sides_without_cot_amplification(host):
    """Sources with a side within 2° of the vertical (drawn from the priors): the error
    stays within 5e-6 of the oracle, as for any other source.  Evaluated term by term,
    the coefficients of order cot β and cot²β turn FP32 rounding into errors up to
    cot²β · 2⁻²⁴ (0.2 at 0.03°); with the logarithms combined it was still ~7e-6 · cot β."""
    g = np.linspace(-20e3, 20e3, 30)
    X, Y = [np.ascontiguousarray(a.ravel()) for a in np.meshgrid(g, g)]
    los = np.ascontiguousarray(np.tile(LOS, (X.size, 1)))
    theta = [th for th in cdm_prior_rows(300, seed=5) if min_vertical_angle(th) < 2.0]
    assert len(theta) >= 8
    for th in theta:
        ref = cdm.los_displacements(th, CDM_LAYOUT, X, Y, los, 0.25)
        out = np.empty(X.size)
        t = np.ascontiguousarray(th, dtype=np.float64)
        assert host.cdm_host_los(_dp(t), X.size, _dp(X), _dp(Y), _dp(los), 0.25, _dp(out)) == 0
        err = np.max(np.abs(out - ref)) / np.max(np.abs(ref))
        assert err <= 5e-6, (min_vertical_angle(th), err)


def test_prior_sources_within_1e5(host):
    """300 prior sources: every one within 5e-6 of the oracle (measured: max 2.2e-6, median
    2.8e-7).  Deep rectangles, whose four sides would cancel to a small fraction of each
    side's value, are integrated by quadrature; near shallow vertices each station takes the
    configuration whose legs point away from it."""
    g = np.linspace(-20e3, 20e3, 30)
    X, Y = [np.ascontiguousarray(a.ravel()) for a in np.meshgrid(g, g)]
    los = np.ascontiguousarray(np.tile(LOS, (X.size, 1)))
    errs = []
    for th in cdm_prior_rows(300, seed=5):
        ref = cdm.los_displacements(th, CDM_LAYOUT, X, Y, los, 0.25)
        out = np.empty(X.size)
        t = np.ascontiguousarray(th, dtype=np.float64)
        assert host.cdm_host_los(_dp(t), X.size, _dp(X), _dp(Y), _dp(los), 0.25, _dp(out)) == 0
        errs.append(np.max(np.abs(out - ref)) / np.max(np.abs(ref)))
    errs = np.array(errs)
    assert errs.max() <= 5e-6, errs.max()
    assert np.median(errs) <= 1e-6, np.median(errs)


def test_exactly_vertical_sides(host):
    """Unrotated or axis-aligned bodies have sides exactly along the vertical, which the
    reference drops (libcdm.py:320-324); the set-up recognises them without acos."""
    g = np.linspace(-20e3, 20e3, 30)
    X, Y = [np.ascontiguousarray(a.ravel()) for a in np.meshgrid(g, g)]
    los = np.ascontiguousarray(np.tile(LOS, (X.size, 1)))
    for omega in ((0.0, 0.0, 0.0), (0.0, 90.0, 0.0), (45.0, 0.0, 0.0)):
        th = np.array([1000.0, -2000.0, 4000.0, 10.0, 800.0, 1200.0, 600.0, *omega])
        ref = cdm.los_displacements(th, CDM_LAYOUT, X, Y, los, 0.25)
        out = np.empty(X.size)
        assert host.cdm_host_los(_dp(th), X.size, _dp(X), _dp(Y), _dp(los), 0.25, _dp(out)) == 0
        assert np.max(np.abs(out - ref)) <= 1e-5 * np.max(np.abs(ref)), omega
