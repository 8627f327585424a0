// CDM per-side arithmetic: FP64 set-up of the 12 angular-dislocation pairs of
// a chain (corners, frames, coefficients) and the FP32 evaluation of one pair
// at a group of stations.  Used by the likelihood kernels in forward.cu; the
// functions are plain inline code so that the same source can also be compiled
// for the host to study its rounding.
//
// Reference: models/cdm/cdm/libcdm.py:174-242 (corners, active rectangles),
// libcdm.py:310-372 (angular-dislocation pair of one side, artefact-free
// configurations I and II), libcdm.py:375-430 (AngDisDisp terms).
//
// A rectangle far from the stations compared with its size (far from the free
// surface, or far from a tile of stations) is evaluated instead as the integral of
// point tensile dislocations over its area (Gauss-Legendre product rule, RectQ
// below): the same field without the cancellation between its four sides, and
// with a few nodes where the stations are far.
#pragma once
#include <math.h>
#include <stdint.h>

#include "gauss_legendre.cuh"

#ifndef AG_DEVICE_INLINE
#define AG_DEVICE_INLINE __device__ __forceinline__
#endif
#ifndef AG_CDM_FN
#define AG_CDM_FN __device__ inline
#endif

namespace ag {

constexpr int kSides = 12;

// ---------------------------------------------------------------------------
// per-side constants of one angular-dislocation pair (48 floats).  β is the
// angle of the side from the downward vertical; "configuration II" values,
// the per-station sign sg = -1 of configuration I (β - π) is applied in the
// pair evaluation.  Coefficients of the two log differences carry ln 2 (the
// logs are evaluated in base 2) and those of the Burgers-function difference
// carry the factor 2 of Fi = 2 atan2(...).
//
// Near-vertical ("steep") sides, |cot β| >= kSteepCot: several coefficients grow
// like cot β and cot²β while the combinations they multiply are O(β); evaluated
// term by term they cancel and FP32 rounding (of the terms and of the side
// constants) is amplified by up to cot²β.  These sides take their own evaluation
// (side_pair_t with Steep = true): the ratio configuration at every station, and the
// cancelling groups rewritten as remainders computed without cancellation, with
// O(1) coefficients (derivation in side_pair_t).
struct __align__(16) SideC {
    float4 q[12];
};
// q0: c, s, k1, k2            frame (unit horizontal side direction) and vertex A
// q1: dy1, aA, aB, da         y1(B) - y1(A); depths of A and B; aB - aA
// q2: sb, cb, tb2, ctb2       sin β, cos β, tan(β/2), cot(β/2)
// q3: daS, C1F, C2F, C3F      da·(aA+aB); 2 × coefficients of ΔFi
// q4: C1P, C2P, kc1, kc2      ln 2 × coefficients of Δlog(r+a); k·cot·b1, k·cot·b2
// q5: nb1, nb2, hb1, hb2      2ν b1, 2ν b2, k b1/2, k b2/2
// q6: b1, b2, C1m10, C3m10
// q7: C1Q, C2Q, C3Q, C1m11    ln 2 × configuration-signed coefficients of Δlog(r-z3)
// q8: C3m11, C1m12, aAsb, naAcb   aA·sin β, -aA·cos β
// q9: dz1, dz3, kc2L, omc     Δz1, Δz3 (configuration II); ln 2 · kc2; 1 - |cos β|
// q10: a1c, dc, ssb, cot      steep sides: aA·omc, Δc, sign(cos β)·sin β, cot β
// q11: kr1, kr2, t, ct2       steep sides: k cot β b2, k cot β b1, tan(β'/2), cot(β'/2)
//                             (β' the ratio-configuration angle)
constexpr double kSteepCot = 3.0;

// Per-side constant by its position in SideC (q[i >> 2], component i & 3)
enum : int {
    K_C = 0, K_S, K_K1, K_K2, K_DY1, K_AA, K_AB, K_DA, K_SB, K_CB, K_TB2, K_CTB2, K_DAS, K_C1F, K_C2F, K_C3F,
    K_C1P, K_C2P, K_KC1, K_KC2, K_NB1, K_NB2, K_HB1, K_HB2, K_B1, K_B2, K_C1M10, K_C3M10, K_C1Q, K_C2Q, K_C3Q,
    K_C1M11, K_C3M11, K_C1M12, K_AASB, K_NAACB, K_DZ1, K_DZ3, K_KC2L, K_OMC, K_A1C, K_DC, K_SSB, K_COT,
    K_KR1, K_KR2, K_T, K_CT2
};

// ---------------------------------------------------------------------------
// FP64 per-chain set-up: rotation, corners, geometry check, per-side constants
struct Vec3 { double x, y, z; };
AG_CDM_FN Vec3 v_sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
AG_CDM_FN Vec3 v_add(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
AG_CDM_FN Vec3 v_scale(Vec3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
AG_CDM_FN Vec3 v_cross(Vec3 a, Vec3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
AG_CDM_FN double v_dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

AG_CDM_FN void split_hilo(double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// Whether a side takes part and whether it is near-vertical.  Vertical sides contribute
// nothing (libcdm.py:320-324: |β| or |π - β| below the double epsilon, i.e. cos β = ±1
// exactly; acos of the next double below 1 is already 1.5e-8).
AG_CDM_FN void side_class(Vec3 pa, Vec3 pb, bool& active, bool& steep) {
    const Vec3 side = v_sub(pb, pa);
    const double L = sqrt(v_dot(side, side));
    const double iL = 1.0 / L;
    const double cb = -side.z * iL;
    active = (L > 0.0) && (fabs(cb) < 1.0);
    steep = false;
    if (active) {
        const double sb = sqrt(side.x * side.x + side.y * side.y) * iL;
        steep = fabs(cb * (1.0 / sb)) >= kSteepCot;
    }
}

// Constants of an active side (side_class: active); steep selects the near-vertical set
AG_CDM_FN void fill_side(SideC& S, Vec3 pa, Vec3 pb, Vec3 bvec, double nu, double x0, double y0, bool steep) {
    const double PI = 3.14159265358979323846;
    const double LN2 = 0.69314718055994530942;
    Vec3 side = v_sub(pb, pa);
    double L = sqrt(v_dot(side, side));
    const double iL = 1.0 / L;
    double cb = -side.z * iL;                        // cos β, β in [0, π]
    double hl = sqrt(side.x * side.x + side.y * side.y);
    const double ihl = 1.0 / hl;
    double c = side.x * ihl, s = side.y * ihl;       // e1 = (c, s, 0), e2 = (s, -c, 0)
    double sb = hl * iL;                             // sin β >= 0
    const double isb = 1.0 / sb;
    const double i1pc = 1.0 / (1.0 + fabs(cb));      // no cancellation in 1 + |cos β|
    // tan(β/2) = sin β/(1 + cos β) = (1 - cos β)/sin β, cot(β/2) its inverse
    double tb2 = (cb >= 0.0) ? sb * i1pc : (1.0 - cb) * isb;
    double ctb2 = (cb >= 0.0) ? (1.0 + cb) * isb : sb * i1pc;
    double cot = cb * isb;
    double k = 1.0 - 2.0 * nu;
    double rx = pa.x - x0, ry = pa.y - y0;
    double k1 = c * rx + s * ry;
    double k2 = s * rx - c * ry;
    double aA = -pa.z, aB = -pb.z, da = aB - aA;
    double dy1 = -hl;                                // y1(B) - y1(A) = -e1·side
    // slip in the angular-dislocation frame, with the 1/(2π) of the formula folded in
    const double inv2pi = 0.5 / PI;
    double b1 = (c * bvec.x + s * bvec.y) * inv2pi;
    double b2 = (s * bvec.x - c * bvec.y) * inv2pi;
    double b3 = -bvec.z * inv2pi;
    double kc1 = k * cot * b1, kc2 = k * cot * b2;
    double C1F = b1 * (1.0 - k * cot * cot);
    double C2F = b2 * (1.0 + k * cot * cot);
    double C3F = kc1 + b3;
    double C1P = -b2 * k * (0.5 - cot * cot);
    double C2P = b1 * k * (0.5 + cot * cot);
    double C1m10 = -b1 * sb * cb + b3 * sb * sb;
    double C3m10 = -b1 * cb * cb + b3 * sb * cb;
    double C1Q = -kc2 * cot * cb;
    double C2Q = -kc1 * isb;
    double C3Q = kc2 * cb;
    double C1m11 = b2 * sb;
    double C3m11 = b2 * cb;
    double C1m12 = b1 * cb - b3 * sb;
    S.q[0] = make_float4((float)c, (float)s, (float)k1, (float)k2);
    S.q[1] = make_float4((float)dy1, (float)aA, (float)aB, (float)da);
    S.q[2] = make_float4((float)sb, (float)cb, (float)tb2, (float)ctb2);
    S.q[3] = make_float4((float)(da * (aA + aB)), (float)(2.0 * C1F), (float)(2.0 * C2F), (float)(2.0 * C3F));
    S.q[4] = make_float4((float)(LN2 * C1P), (float)(LN2 * C2P), (float)kc1, (float)kc2);
    S.q[5] = make_float4((float)(2.0 * nu * b1), (float)(2.0 * nu * b2), (float)(0.5 * k * b1),
                         (float)(0.5 * k * b2));
    S.q[6] = make_float4((float)b1, (float)b2, (float)C1m10, (float)C3m10);
    S.q[7] = make_float4((float)(LN2 * C1Q), (float)(LN2 * C2Q), (float)(LN2 * C3Q), (float)C1m11);
    S.q[8] = make_float4((float)C3m11, (float)C1m12, (float)(aA * sb), (float)(-aA * cb));
    const double omc = sb * sb * i1pc;               // 1 - |cos β| without cancellation
    const double sgn = (cb >= 0.0) ? 1.0 : -1.0;
    S.q[9] = make_float4((float)(dy1 * cb + da * sb), (float)(dy1 * sb - da * cb), (float)(LN2 * kc2), (float)omc);
    S.q[10] = make_float4(0.f, 0.f, 0.f, 0.f);
    S.q[11] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (steep) {
        // ratio configuration: β' = β if cos β > 0, β - π otherwise; t = tan(β'/2)
        const double t = (cb > 0.0) ? tb2 : -ctb2;
        S.q[3].y = (float)(2.0 * b1);                  // ΔFi: the k cot²β parts are in R_F
        S.q[3].z = (float)(2.0 * b2);
        S.q[4].x = (float)(-LN2 * 0.5 * k * b2);       // v1: -k b2/2 · Δlog(r+a)
        S.q[4].y = (float)(LN2 * 0.5 * k * b1);        // v2: k b1/2 · Δlog(r+a)
        S.q[7].y = (float)(-LN2 * k * b1 * cb);        // v2: -sg k b1 cos β · Δlog(r-z3)
        S.q[10] = make_float4((float)(aA * omc), (float)(da * omc + sgn * dy1 * sb), (float)(sgn * sb),
                              (float)cot);
        S.q[11] = make_float4((float)(k * cot * b2), (float)(k * cot * b1), (float)t,
                              (float)((cb > 0.0) ? ctb2 : -tb2));
    }
}

// corners of the three rectangles (libcdm.py:174-217); returns true if any is above the surface
template <class Layout>
AG_CDM_FN bool cdm_corners(const double* th, const Layout& L, Vec3 V[3][4]) {
    const double x0 = th[L.x_idx], y0 = th[L.x_idx + 1], depth = th[L.depth_idx];
    const double lx = 2.0 * th[L.axes_idx], ly = 2.0 * th[L.axes_idx + 1],
                 lz = 2.0 * th[L.axes_idx + 2];
    double sx, cx, sy, cy, sz, cz;
    sincospi(th[L.omega_idx] / 180.0, &sx, &cx);
    sincospi(th[L.omega_idx + 1] / 180.0, &sy, &cy);
    sincospi(th[L.omega_idx + 2] / 180.0, &sz, &cz);
    // R = Rz·Ry·Rx with Rx = [[1,0,0],[0,cx,sx],[0,-sx,cx]], Ry = [[cy,0,-sy],[0,1,0],[sy,0,cy]],
    // Rz = [[cz,sz,0],[-sz,cz,0],[0,0,1]]; columns ex, ey, ez are the body axes in EFCS
    const double ryx[3][3] = {{cy, sy * sx, -sy * cx},   // Ry·Rx
                              {0.0, cx, sx},
                              {sy, cy * -sx, cy * cx}};
    double R[3][3];
    const double rz[3][3] = {{cz, sz, 0.0}, {-sz, cz, 0.0}, {0.0, 0.0, 1.0}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            R[i][j] = rz[i][0] * ryx[0][j] + rz[i][1] * ryx[1][j] + rz[i][2] * ryx[2][j];
    Vec3 ex{R[0][0], R[1][0], R[2][0]}, ey{R[0][1], R[1][1], R[2][1]}, ez{R[0][2], R[1][2], R[2][2]};
    Vec3 c0{x0, y0, -depth};
    Vec3 p1 = v_add(c0, v_add(v_scale(ey, 0.5 * ly), v_scale(ez, 0.5 * lz)));
    Vec3 p2 = v_sub(p1, v_scale(ey, ly));
    Vec3 p3 = v_sub(p2, v_scale(ez, lz));
    Vec3 p4 = v_sub(p1, v_scale(ez, lz));
    Vec3 q1 = v_add(v_sub(c0, v_scale(ex, 0.5 * lx)), v_scale(ez, 0.5 * lz));
    Vec3 q2 = v_add(q1, v_scale(ex, lx));
    Vec3 q3 = v_sub(q2, v_scale(ez, lz));
    Vec3 q4 = v_sub(q1, v_scale(ez, lz));
    Vec3 r1 = v_add(c0, v_add(v_scale(ex, 0.5 * lx), v_scale(ey, 0.5 * ly)));
    Vec3 r2 = v_sub(r1, v_scale(ex, lx));
    Vec3 r3 = v_sub(r2, v_scale(ey, ly));
    Vec3 r4 = v_sub(r1, v_scale(ey, ly));
    V[0][0] = p1; V[0][1] = p2; V[0][2] = p3; V[0][3] = p4;
    V[1][0] = q1; V[1][1] = q2; V[1][2] = q3; V[1][3] = q4;
    V[2][0] = r1; V[2][1] = r2; V[2][2] = r3; V[2][3] = r4;
    bool above = false;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 4; ++b) above |= (V[a][b].z > 0.0);
    return above;
}

// ---------------------------------------------------------------------------
// Far-field rectangles: quadrature of point tensile dislocations.
//
// A rectangle of uniform opening is the superposition of point tensile dislocations
// over its area, each with the half-space surface displacement of Okada (1985, BSSA
// 75(4), point source, tensile component): in the strike frame of the plane (x along
// strike, the plane dipping by δ towards -y), for a point at depth d and a station at
// horizontal offset (x, y),
//     R² = x² + y² + d²,  q = y sin δ - d cos δ,  k = 1 - 2ν,
//     I1 = k y [1/(R(R+d)²) - x²(3R+d)/(R³(R+d)³)],  I2 = the same with x and y swapped,
//     I3 = k x/R³ - I2,  I5 = k [1/(R(R+d)) - x²(2R+d)/(R³(R+d)²)],
//     (ux, uy, uz) = P/(2π) (3x q²/R⁵ - I3 sin²δ, 3y q²/R⁵ - I1 sin²δ, 3d q²/R⁵ - I5 sin²δ)
// for potency P (opening × area).  (Its sign convention agrees with the angular-dislocation
// rectangles of libcdm.py:250-273, of which it is the limit for a vanishing rectangle;
// checked in the CPU tests.)  q is the same for every point of the plane.
//
// The rectangle's field is the integral of that kernel over the rectangle, taken with an
// n1 × n2 Gauss-Legendre product rule.  The integrand is analytic in each coordinate; its
// singularities lie where the station-to-point distance vanishes, at least D from every
// point of the rectangle for the stations in question, so the error of an n-point rule
// along a side of half-length h falls like ρ^(-2n), ρ = D/h + sqrt((D/h)² + 1) (the
// Bernstein ellipse through the nearest singularity).  Each direction gets the smallest n
// with ρ^(-2n) <= kQuadTol, found by comparing δ² = (D/h)² with the thresholds
// kQuadDelta2 (no transcendental function, so the kernel, the work count and the host
// build decide alike).  Two distances are used:
//   * per chain, D = the depth of the rectangle's shallowest corner (a lower bound for every
//     station): a rectangle with n1 n2 <= kQuadBudget is integrated everywhere ("far"
//     rectangle; its four sides cost about as much as 20 nodes), the others are evaluated
//     by their sides;
//   * per station tile (AG_STATION_TILE consecutive stations), D² = depth² + gap², gap the
//     horizontal distance between the tile's bounding box and the rectangle's corners': far
//     rectangles take the tile's (smaller) node counts, and a rectangle evaluated by its
//     sides is integrated over the tiles where n1 n2 <= kQuadBudget nodes cost less than
//     its sides.  Stations far from the source then take a few nodes instead of many.
// The nodes are summed in FP32 without cancellation: for a rectangle whose distance from
// the stations is many times its size, the FP32 sum of its four sides loses the factor
// distance/size in accuracy, the quadrature does not.
constexpr double kQuadTol = 1e-7;
constexpr int kQuadBudget = 32;

// δ_n² = ((ρ_n - 1/ρ_n)/2)², ρ_n = kQuadTol^(-1/(2n)): n nodes per direction suffice for
// δ² >= δ_n² (n = 1 ... kGaussMax; rounded up to FP32)
AG_GL_TABLE float kQuadDelta2[kGaussMax] = {
    2.499999750e+06f, 7.900695190e+02f, 5.336203003e+01f, 1.356297970e+01f, 5.789669037e+00f, 3.186530590e+00f,
    2.025000095e+00f, 1.408073664e+00f, 1.040413141e+00f, 8.028496504e-01f, 6.399435997e-01f, 5.230506659e-01f,
    4.361335039e-01f, 3.696263731e-01f, 3.175248802e-01f, 2.758984566e-01f};

// smallest n in 1 ... kGaussMax with δ² >= δ_n², kGaussMax + 1 if none: the number of
// thresholds above δ² (they decrease with n), by binary search
template <class F>
AG_CDM_FN int quad_n(F delta2) {
    int k = 0;
    for (int step = 8; step > 0; step >>= 1)
        if (k + step <= kGaussMax && delta2 < (F)kQuadDelta2[k + step - 1]) k += step;
    return k + 1;
}

// A rectangle's quadrature in parametric form; the nodes of an n1 × n2 rule are generated
// from it where they are used (rect_node)
struct __align__(16) RectQ {
    float4 h0;    // strike direction (a, b) = (cos, sin), sin δ, q offset Q0
    float4 h1;    // -k sin²δ, 1/h1², 1/h2², D² (D: depth of the shallowest corner)
    float4 c;     // centre in the strike frame (relative to the source centre), its depth, weight scale
    float4 e1;    // half edge P2 - P1 in the strike frame (x, y, depth); FLOP per station of the sides
    float4 e2;    // half edge P4 - P1 in the strike frame (x, y, depth); chain node counts n1 + 256 n2
    float4 box;   // the corners' horizontal bounding box relative to the source centre: x0, x1, y0, y1
};

// Per-chain plan shared by the set-up kernel and the work count: bits 0-11 sides evaluated
// as angular-dislocation pairs (where the tile does not integrate their rectangle), 12-23
// which of them are near-vertical, 24-26 far rectangles integrated everywhere (their node
// counts in nq), 27-29 rectangles that take part (a RectQ each).  Rectangles that take part
// follow libcdm.py:226-242 (a zero semi-axis leaves only the rectangle spanned by the other
// two).
template <class Layout>
AG_CDM_FN uint32_t cdm_plan(const double* th, const Layout& L, const Vec3 V[3][4], int nq[3][2]) {
    const double ax = th[L.axes_idx], ay = th[L.axes_idx + 1], az = th[L.axes_idx + 2];
    bool use[3];
    if (ax == 0.0 && ay == 0.0 && az == 0.0) {
        use[0] = use[1] = use[2] = false;
    } else if (ax == 0.0 && ay != 0.0 && az != 0.0) {
        use[0] = true; use[1] = use[2] = false;
    } else if (ax != 0.0 && ay == 0.0 && az != 0.0) {
        use[1] = true; use[0] = use[2] = false;
    } else if (ax != 0.0 && ay != 0.0 && az == 0.0) {
        use[2] = true; use[0] = use[1] = false;
    } else {
        use[0] = use[1] = use[2] = true;
    }
    uint32_t mask = 0u;
    for (int r = 0; r < 3; ++r) {
        nq[r][0] = nq[r][1] = 0;
        if (!use[r]) continue;
        const Vec3 e1 = v_sub(V[r][1], V[r][0]), e2 = v_sub(V[r][3], V[r][0]);
        const double h1 = 0.5 * sqrt(v_dot(e1, e1)), h2 = 0.5 * sqrt(v_dot(e2, e2));
        double D = -V[r][0].z;
        for (int e = 1; e < 4; ++e) D = fmin(D, -V[r][e].z);
        if (h1 > 0.0 && h2 > 0.0 && D > 0.0) {
            const int n1 = quad_n((D * D) / (h1 * h1)), n2 = quad_n((D * D) / (h2 * h2));
            if (n1 <= kGaussMax && n2 <= kGaussMax && n1 * n2 <= kQuadBudget) {
                nq[r][0] = n1;
                nq[r][1] = n2;
                mask |= (1u << (24 + r)) | (1u << (27 + r));
                continue;
            }
        }
        for (int e = 0; e < 4; ++e) {
            bool act, steep;
            side_class(V[r][e], V[r][(e + 1) & 3], act, steep);
            if (act) mask |= 1u << (r * 4 + e);
            if (act && steep) mask |= 1u << (kSides + r * 4 + e);
        }
        if (mask >> (4 * r) & 0xFu) mask |= 1u << (27 + r);
    }
    return mask;
}

// float rounded down / up (a box that contains the exact one)
AG_CDM_FN float f32_down(double v) {
#ifdef __CUDA_ARCH__
    return __double2float_rd(v);
#else
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
#endif
}
AG_CDM_FN float f32_up(double v) {
#ifdef __CUDA_ARCH__
    return __double2float_ru(v);
#else
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, INFINITY);
    return f;
#endif
}

// FP32 work per station (FMA = 2), counted from the pair and quadrature code below and
// checked against a counting evaluation in the CPU tests
constexpr int kFlopSide = 251;          // one angular-dislocation pair
constexpr int kFlopSteepExtra = 78;     // near-vertical pair: remainders of the cot β terms
constexpr int kFlopQuadRect = 19;       // quadrature rectangle: strike frame, q, back to EFCS
constexpr int kFlopQuadNode = 43;       // one point tensile dislocation, weighted sum
constexpr int kFlopStation = 31;        // coordinates, LOS projection, residual, float-float misfit
constexpr int kSfuSide = 13, kSfuSteepExtra = 3, kSfuQuadNode = 2;

// Parametric quadrature of rectangle P1..P4 (P2 - P1 and P4 - P1 its edges); side_flop is
// the FP32 work per station of its sides (0 for a far rectangle), n1, n2 its node counts
// as a far rectangle (0 otherwise)
AG_CDM_FN void fill_rect(RectQ& R, const Vec3 P[4], double opening, double nu, double x0, double y0,
                         int side_flop, int n1, int n2) {
    const double PI = 3.14159265358979323846;
    const Vec3 e1 = v_sub(P[1], P[0]), e2 = v_sub(P[3], P[0]);
    Vec3 nrm = v_cross(e1, e2);
    const double area = sqrt(v_dot(nrm, nrm));
    nrm = v_scale(nrm, 1.0 / area);
    if (nrm.z < 0.0) nrm = v_scale(nrm, -1.0);      // the field does not depend on the normal's sense
    const double sd = sqrt(nrm.x * nrm.x + nrm.y * nrm.y), cd = nrm.z;
    // strike (a, b): horizontal, perpendicular to the normal's horizontal part, with the
    // plane dipping towards -y of the strike frame (y = (-b, a))
    double a = 1.0, b = 0.0;
    if (sd > 0.0) {
        a = -nrm.y / sd;
        b = nrm.x / sd;
    }
    const Vec3 c = v_add(P[0], v_scale(v_add(e1, e2), 0.5));
    const double cx = c.x - x0, cy = c.y - y0;
    const double yc = -b * cx + a * cy;
    const double h1 = 0.5 * sqrt(v_dot(e1, e1)), h2 = 0.5 * sqrt(v_dot(e2, e2));
    double D = -P[0].z, bx0 = P[0].x, bx1 = P[0].x, by0 = P[0].y, by1 = P[0].y;
    for (int k = 1; k < 4; ++k) {
        D = fmin(D, -P[k].z);
        bx0 = fmin(bx0, P[k].x); bx1 = fmax(bx1, P[k].x);
        by0 = fmin(by0, P[k].y); by1 = fmax(by1, P[k].y);
    }
    R.h0 = make_float4((float)a, (float)b, (float)sd, (float)(yc * sd + (-c.z) * cd));
    R.h1 = make_float4((float)(-(1.0 - 2.0 * nu) * sd * sd), h1 > 0.0 ? (float)(1.0 / (h1 * h1)) : 0.f,
                       h2 > 0.0 ? (float)(1.0 / (h2 * h2)) : 0.f, f32_down(D * D));
    R.c = make_float4((float)(a * cx + b * cy), (float)yc, (float)(-c.z),
                      (float)(0.25 * area * opening / (2.0 * PI)));
    const Vec3 E1 = v_scale(e1, 0.5), E2 = v_scale(e2, 0.5);
    R.e1 = make_float4((float)(a * E1.x + b * E1.y), (float)(-b * E1.x + a * E1.y), (float)(-E1.z), (float)side_flop);
    R.e2 = make_float4((float)(a * E2.x + b * E2.y), (float)(-b * E2.x + a * E2.y), (float)(-E2.z),
                       __int_as_float(n1 + 256 * n2));
    R.box = make_float4(f32_down(bx0 - x0), f32_up(bx1 - x0), f32_down(by0 - y0), f32_up(by1 - y0));
}

// FP32 work per station of the sides of rectangle r in the plan
AG_CDM_FN void rect_side_work(uint32_t mask, int r, int& flop, int& sfu) {
    flop = 0;
    sfu = 0;
    for (int e = 0; e < 4; ++e) {
        const int k = 4 * r + e;
        if (!(mask >> k & 1u)) continue;
        const bool st = (mask >> (kSides + k)) & 1u;
        flop += kFlopSide + (st ? kFlopSteepExtra : 0);
        sfu += kSfuSide + (st ? kSfuSteepExtra : 0);
    }
}

// Constants of a chain whose corners V lie below the surface, following the plan: a RectQ
// for every rectangle that takes part, and the SideC of the active sides of the rectangles
// that are not far.  Returns the plan's mask.
template <class Layout>
AG_CDM_FN uint32_t cdm_sides(const double* th, const Layout& L, const Vec3 V[3][4], double x0, double y0,
                             SideC* side, RectQ* rect) {
    int nq[3][2];
    const uint32_t mask = cdm_plan(th, L, V, nq);
    const double opening = th[L.strength_idx];
    for (int r = 0; r < 3; ++r) {
        if (!(mask >> (27 + r) & 1u)) continue;
        int sf, su;
        rect_side_work(mask, r, sf, su);
        fill_rect(rect[r], V[r], opening, L.nu, x0, y0, sf, nq[r][0], nq[r][1]);
        if (mask >> (24 + r) & 1u) continue;
        Vec3 nrm = v_cross(v_sub(V[r][1], V[r][0]), v_sub(V[r][3], V[r][0]));
        nrm = v_scale(nrm, 1.0 / sqrt(v_dot(nrm, nrm)));
        const Vec3 b = v_scale(nrm, opening);
        for (int e = 0; e < 4; ++e)
            if (mask >> (r * 4 + e) & 1u)
                fill_side(side[r * 4 + e], V[r][e], V[r][(e + 1) & 3], b, L.nu, x0, y0,
                          (mask >> (kSides + r * 4 + e)) & 1u);
    }
    return mask;
}

// The plan and the RectQ of every rectangle that takes part (no side constants): what the
// cost classes and the work count need
template <class Layout>
AG_CDM_FN uint32_t cdm_rects(const double* th, const Layout& L, const Vec3 V[3][4], double x0, double y0,
                             RectQ* rect) {
    int nq[3][2];
    const uint32_t mask = cdm_plan(th, L, V, nq);
    for (int r = 0; r < 3; ++r) {
        if (!(mask >> (27 + r) & 1u)) continue;
        int sf, su;
        rect_side_work(mask, r, sf, su);
        fill_rect(rect[r], V[r], th[L.strength_idx], L.nu, x0, y0, sf, nq[r][0], nq[r][1]);
    }
    return mask;
}

// Node counts of rectangle R over a station tile whose bounding box, relative to the source
// centre, is [bx0, bx1] × [by0, by1]: δ² = (D² + gap²)/h² per direction.  A far rectangle
// keeps at most its chain node counts; a rectangle evaluated by its sides is integrated over
// the tile when its nodes fit the budget and cost less than its sides.  Returns whether the
// tile integrates it.
AG_CDM_FN bool tile_quad(const RectQ& R, bool far, float bx0, float bx1, float by0, float by1, int& n1, int& n2) {
    const float gx = fmaxf(0.0f, fmaxf(__fsub_rn(R.box.x, bx1), __fsub_rn(bx0, R.box.y)));
    const float gy = fmaxf(0.0f, fmaxf(__fsub_rn(R.box.z, by1), __fsub_rn(by0, R.box.w)));
    const float D2 = __fadd_rn(R.h1.w, __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)));
    n1 = quad_n(__fmul_rn(D2, R.h1.y));
    n2 = quad_n(__fmul_rn(D2, R.h1.z));
    if (far) {
        const int nc = __float_as_int(R.e2.w);
        n1 = n1 < (nc & 255) ? n1 : (nc & 255);
        n2 = n2 < (nc >> 8) ? n2 : (nc >> 8);
        return true;
    }
    return n1 <= kGaussMax && n2 <= kGaussMax && n1 * n2 <= kQuadBudget &&
           kFlopQuadRect + kFlopQuadNode * n1 * n2 < (int)R.e1.w;
}

// Node k = (i, j) of the n1 × n2 rule on R (k < n1 n2 <= kQuadBudget): position in the
// strike frame, depth, weight, from the FP32 rules gx, gw (kGaussXf, kGaussWf or a copy).
// i = floor((k + 1/2)/n2) is exact in FP32 for k < 32 (the fraction stays 1/(2 n2) away from
// an integer, far above the rounding of the approximate reciprocal).
AG_CDM_FN float4 rect_node(const RectQ& R, int n1, int n2, int k, const float* gx, const float* gw) {
    const int i = (int)(__fmul_rn(__fadd_rn((float)k, 0.5f), __fdividef(1.0f, (float)n2)));
    const int j = k - i * n2;
    const float s = gx[gauss_offset(n1) + i], t = gx[gauss_offset(n2) + j];
    const float w = __fmul_rn(gw[gauss_offset(n1) + i], gw[gauss_offset(n2) + j]);
    return make_float4(fmaf(t, R.e2.x, fmaf(s, R.e1.x, R.c.x)), fmaf(t, R.e2.y, fmaf(s, R.e1.y, R.c.y)),
                       fmaf(t, R.e2.z, fmaf(s, R.e1.z, R.c.z)), __fmul_rn(w, R.c.w));
}

// FP32 work per station of a chain over one tile (its plan's sides, and the nodes of the
// rectangles the tile integrates)
AG_CDM_FN void tile_work(const RectQ* rect, uint32_t mask, float bx0, float bx1, float by0, float by1,
                         uint32_t& flop, uint32_t& sfu) {
    uint32_t f = kFlopStation, u = 0;
    for (int r = 0; r < 3; ++r) {
        if (!(mask >> (27 + r) & 1u)) continue;
        int n1, n2;
        if (tile_quad(rect[r], (mask >> (24 + r)) & 1u, bx0, bx1, by0, by1, n1, n2)) {
            f += kFlopQuadRect + kFlopQuadNode * n1 * n2;
            u += kSfuQuadNode * n1 * n2;
        } else {
            int sf, su;
            rect_side_work(mask, r, sf, su);
            f += sf;
            u += su;
        }
    }
    flop = f;
    sfu = u;
}

// ---------------------------------------------------------------------------
// FP32 elementary functions (own implementations)

AG_DEVICE_INLINE float fast_rcp(float x) { return __fdividef(1.0f, x); }

// log2(ρ) of a ratio ρ > 0 given s = (ρ - 1)/(ρ + 1), which the caller forms
// from a difference without cancellation.  For ρ in [√½, √2] (|s| <= 3 - 2√2)
// log2 ρ = 2 atanh(s)/ln 2 = (2/ln 2)(s + s³/3 + s⁵/5 + s⁷/7 + s⁹/9) + O(s¹¹),
// truncation < 2e-9 relative, so ratios near 1 keep full relative accuracy;
// outside that range |log2 ρ| >= 0.5 and the hardware base-2 logarithm of ρ
// (absolute error <= 2^-22.6 on [0.5, 2], 2 ulp elsewhere) is used.
AG_DEVICE_INLINE float log2_ratio(float s, float rho) {
    const float t = __fmul_rn(s, s);
    float p = fmaf(t, 3.205988980e-01f, 4.121985831e-01f);
    p = fmaf(p, t, 5.770780164e-01f);
    p = fmaf(p, t, 9.617966939e-01f);
    p = fmaf(p, t, 2.885390082e+00f);
    const float near = __fmul_rn(s, p);
    return fabsf(s) <= 0.17157288f ? near : __log2f(rho);
}

// atan2(y, x): octant reduction to t = min/max in [0, 1], atan(t) = t·P(t²) with
// P of degree 8, coefficients fitted here by iteratively reweighted least squares
// on the relative error over [0, 1] (<= 1.9 ulp in FP32 Horner form), then
// π/2 - r, π - r and the sign of y restore the quadrant.  atan2(0, 0) = 0; for
// |x|, |y| above 1e-23 the offset in the reciprocal does not change the result.
AG_DEVICE_INLINE float atan2_poly(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float t = mn * fast_rcp(mx + 1e-30f);      // the tiny offset makes atan2(0, 0) = 0
    const float u = t * t;
    float p = 2.903841436e-03f;
    p = fmaf(p, u, -1.628421992e-02f);
    p = fmaf(p, u, 4.304145649e-02f);
    p = fmaf(p, u, -7.533866167e-02f);
    p = fmaf(p, u, 1.065477580e-01f);
    p = fmaf(p, u, -1.420716196e-01f);
    p = fmaf(p, u, 1.999305785e-01f);
    p = fmaf(p, u, -3.333309293e-01f);
    p = fmaf(p, u, 1.0f);
    float r = p * t;
    r = (ay > ax) ? 1.57079632679f - r : r;
    r = (x < 0.0f) ? 3.14159265359f - r : r;
    return copysignf(r, y);
}

// ---------------------------------------------------------------------------
// Arithmetic of side_pair.  Every product that feeds a sum is written as an
// explicit FMA and the remaining adds and multiplies use the non-contracting
// round-to-nearest forms, so the rounding of each operation is fixed by the
// source rather than by the compiler's contraction choices.  (A two-station
// form with packed FP32x2 instructions was measured 2-4% slower on this kernel:
// the FMA pipe throttles the packed instructions, and it was removed.)
AG_DEVICE_INLINE float vfma(float a, float b, float c) { return fmaf(a, b, c); }
AG_DEVICE_INLINE float vadd(float a, float b) { return __fadd_rn(a, b); }
AG_DEVICE_INLINE float vsub(float a, float b) { return __fsub_rn(a, b); }
AG_DEVICE_INLINE float vmul(float a, float b) { return __fmul_rn(a, b); }
AG_DEVICE_INLINE float vneg(float a) { return -a; }
AG_DEVICE_INLINE bool vge0(float a) { return a >= 0.0f; }
AG_DEVICE_INLINE bool vgt0(float a) { return a > 0.0f; }
AG_DEVICE_INLINE bool vand(bool a, bool b) { return a && b; }
AG_DEVICE_INLINE float vsel(bool c, float a, float b) { return c ? a : b; }
AG_DEVICE_INLINE float frcp(float x) { return fast_rcp(x); }
AG_DEVICE_INLINE float vrsqrt(float x) { return rsqrtf(x); }
AG_DEVICE_INLINE float vlog2r(float s, float rho) { return log2_ratio(s, rho); }
AG_DEVICE_INLINE float vatan2(float y, float x) { return atan2_poly(y, x); }

// Several stations per lane as a group of scalars: every operation is the scalar one
// on each element, so results are identical to the one-station form, while the
// independent chains of dependent instructions interleave (instruction-level
// parallelism for the MUFU and FMA latencies) and each side constant is loaded from
// shared memory once for the whole group.
template <int N>
struct SV {
    float v[N];
    AG_DEVICE_INLINE SV() {}
    AG_DEVICE_INLINE SV(float x) {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = x;
    }
};
template <int N>
struct CV { bool v[N]; };
#define AG_SV_MAP(expr)                  \
    SV<N> r;                             \
    _Pragma("unroll") for (int i = 0; i < N; ++i) r.v[i] = (expr); \
    return r
#define AG_CV_MAP(expr)                  \
    CV<N> r;                             \
    _Pragma("unroll") for (int i = 0; i < N; ++i) r.v[i] = (expr); \
    return r
template <int N> AG_DEVICE_INLINE SV<N> vfma(SV<N> x, SV<N> y, SV<N> z) { AG_SV_MAP(fmaf(x.v[i], y.v[i], z.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vadd(SV<N> x, SV<N> y) { AG_SV_MAP(__fadd_rn(x.v[i], y.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vsub(SV<N> x, SV<N> y) { AG_SV_MAP(__fsub_rn(x.v[i], y.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vmul(SV<N> x, SV<N> y) { AG_SV_MAP(__fmul_rn(x.v[i], y.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vneg(SV<N> x) { AG_SV_MAP(-x.v[i]); }
template <int N> AG_DEVICE_INLINE CV<N> vge0(SV<N> x) { AG_CV_MAP(x.v[i] >= 0.0f); }
template <int N> AG_DEVICE_INLINE CV<N> vgt0(SV<N> x) { AG_CV_MAP(x.v[i] > 0.0f); }
template <int N> AG_DEVICE_INLINE CV<N> vand(CV<N> x, CV<N> y) { AG_CV_MAP(x.v[i] && y.v[i]); }
template <int N> AG_DEVICE_INLINE SV<N> vsel(CV<N> c, SV<N> x, SV<N> y) { AG_SV_MAP(c.v[i] ? x.v[i] : y.v[i]); }
template <int N> AG_DEVICE_INLINE SV<N> frcp(SV<N> x) { AG_SV_MAP(fast_rcp(x.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vrsqrt(SV<N> x) { AG_SV_MAP(rsqrtf(x.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vlog2r(SV<N> s, SV<N> rho) { AG_SV_MAP(log2_ratio(s.v[i], rho.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vatan2(SV<N> y, SV<N> x) { AG_SV_MAP(atan2_poly(y.v[i], x.v[i])); }
#undef AG_SV_MAP
#undef AG_CV_MAP

struct ScalarSide {
    float4 q[12];
    AG_DEVICE_INLINE explicit ScalarSide(const SideC& S) {
#pragma unroll
        for (int i = 0; i < 12; ++i) q[i] = S.q[i];
    }
    template <int I>
    AG_DEVICE_INLINE float at() const {
        const float4 t = q[I >> 2];
        return (I & 3) == 0 ? t.x : (I & 3) == 1 ? t.y : (I & 3) == 2 ? t.z : t.w;
    }
    template <int I>
    AG_DEVICE_INLINE float neg() const { return -at<I>(); }
};

#define KC(i) V(k.template at<i>())
#define KN(i) V(k.template neg<i>())

// ---------------------------------------------------------------------------
// One angular-dislocation pair in difference arithmetic: every quantity is
// carried as (value at A, difference B - A), the difference propagated by exact
// identities (Δ(uv) = Δu·v_B + u_A·Δv, Δ(1/u) = -Δu/(u_A u_B),
// Δr = Δ(r²)/(r_A + r_B), Δlog u from s = Δu/(u_A + u_B), the Burgers-function
// difference as one atan2 of the rotation from A to B), so the v(B) - v(A)
// cancellation of the reference formula never happens in floating point.
template <bool Steep, class V, class K>
AG_DEVICE_INLINE void side_pair_t(const K& k, V Xr, V Yr, V& ue, V& un, V& uv) {
    const V c = KC(K_C), s = KC(K_S);
    const V dy1 = KC(K_DY1), aA = KC(K_AA), aB = KC(K_AB), da = KC(K_DA);
    // station in the angular-dislocation frame of vertex A; y2 is the same at B
    const V y1A = vfma(c, Xr, vfma(s, Yr, KN(K_K1)));
    const V y2 = vfma(s, Xr, vfma(KN(K_C), Yr, KN(K_K2)));
    const V y1B = vadd(y1A, dy1);
    // Artefact-free configuration: II (β) or I (β - π; sin, cos and cot(β/2) of β - π are
    // those of β times -1), libcdm.py:342-362.  Both give the same pair away from the other's
    // singular ray (where r - z3 vanishes at the surface); the reference picks I where
    // y1A >= 0.  Here each station takes the configuration whose legs point away from it:
    // with u = y1 sin β - a cos β (z3 of configuration II; u_B = u_A + Δz3, Δz3 = -L), II if
    // u_A + u_B <= 0, else I, so z3 <= 0 and r - z3 >= r at both vertices whenever the
    // station's projection on the side's line falls outside the side.  The reference's rule
    // can leave a leg pointing at a station near a shallow vertex, where r - z3 << r and the
    // large terms cancel in FP32.  A near-vertical side takes the ratio configuration
    // (sg = sign cos β) at every station: its r - z3 has no zero and its Burgers-function
    // argument no sign change at the free surface.
    V sg, ct2;
    const V u3A = vfma(y1A, KC(K_SB), KC(K_NAACB));
    if constexpr (Steep) {
        sg = V(k.template at<K_CB>() > 0.0f ? 1.0f : -1.0f);
        ct2 = KC(K_CT2);
    } else {
        const auto conf1 = vgt0(vfma(V(2.0f), u3A, KC(K_DZ3)));
        sg = vsel(conf1, V(-1.0f), V(1.0f));
        ct2 = vsel(conf1, KN(K_TB2), KC(K_CTB2));
    }
    const V y22 = vmul(y2, y2);
    // r (rA = r2A·irA enters every sum through an FMA)
    const V r2A = vfma(y1A, y1A, vfma(aA, aA, y22));
    const V r2B = vfma(y1B, y1B, vfma(aB, aB, y22));
    const V irA = vrsqrt(r2A), irB = vrsqrt(r2B);
    const V rB = vmul(r2B, irB);
    const V dr = vmul(vfma(dy1, vadd(y1A, y1B), KC(K_DAS)), frcp(vfma(r2A, irA, rB)));
    const V ndir = vmul(vmul(dr, irA), irB);           // -Δ(1/r)
    // r + a
    const V pA = vfma(r2A, irA, aA), pB = vfma(r2B, irB, aB), dp = vadd(dr, da);
    const V ipA = frcp(pA), ipB = frcp(pB);
    const V ndip = vmul(vmul(dp, ipA), ipB);           // -Δ(1/(r+a))
    // z1 = sg (y1 cos β + a sin β), z3 = sg (y1 sin β - a cos β); Δz1, Δz3 are side constants
    const V z1A = vmul(sg, vfma(y1A, KC(K_CB), KC(K_AASB)));
    const V dz1 = vmul(sg, KC(K_DZ1));
    const V z1B = vadd(z1A, dz1);
    const V z3A = vmul(sg, u3A);
    const V dz3 = vmul(sg, KC(K_DZ3));
    const V z3B = vadd(z3A, dz3);
    // r - z3, cancellation-free: (z1² + y2²)/(r + z3) when z3 > 0, else (r + z3) - 2 z3
    const auto posA = vgt0(z3A), posB = vgt0(z3B);
    const V NA = vfma(z1A, z1A, y22), NB = vfma(z1B, z1B, y22);
    const V DA = vfma(r2A, irA, z3A), DB = vfma(r2B, irB, z3B);
    const V uA = vsel(posA, NA, vfma(V(-2.0f), z3A, DA)), vA = vsel(posA, DA, V(1.0f));
    const V uB = vsel(posB, NB, vfma(V(-2.0f), z3B, DB)), vB = vsel(posB, DB, V(1.0f));
    const V iuA = frcp(uA), iuB = frcp(uB);
    const V iqA = vmul(vA, iuA), iqB = vmul(vB, iuB);
    const V dN = vmul(dz1, vadd(z1A, z1B));
    // both in the quotient form: Δq = (ΔN·D_A - N_A·ΔD)/(D_A D_B), ΔD = Δr + Δz3
    const V dq = vsel(vand(posA, posB), vmul(vfma(dN, DA, vneg(vmul(NA, vadd(dr, dz3)))), frcp(vmul(DA, DB))),
                      vsub(dr, dz3));
    const V ndiq = vmul(vmul(dq, iqA), iqB);           // -Δ(1/q)
    // log differences, base 2: s = Δu/(u_A + u_B) and the ratio u_B/u_A
    const V dLp = vlog2r(vmul(dp, frcp(vadd(pA, pB))), vmul(pB, ipA));
    const V xq = vmul(dq, iqA);                        // Δq/q_A
    const V dLq = vlog2r(vmul(xq, frcp(vadd(V(2.0f), xq))), vadd(V(1.0f), xq));
    // Burgers function difference: rotation of (x, y2) from A to B; y2 keeps its sign so
    // the rotation never crosses atan2's cut (the factor 2 is in the coefficients)
    const V xA = vfma(pA, ct2, vneg(y1A));
    const V dx = vfma(dp, ct2, KN(K_DY1));
    const V xB = vadd(xA, dx);
    const V dF = vatan2(vmul(vneg(y2), dx), vfma(xA, xB, y22));
    // monomials: value at A, value at B, difference
    const V m1B = vmul(y2, ipB), ndm1 = vmul(y2, ndip);
    const V m2A = vmul(y1A, ipA), m2B = vmul(y1B, ipB);
    const V dm2 = vfma(dy1, ipB, vneg(vmul(y1A, ndip)));
    const V dm3 = vfma(da, ipB, vmul(KN(K_AA), ndip));
    const V dm4 = vfma(dm2, m1B, vneg(vmul(m2A, ndm1)));
    const V dm35 = vfma(dm2, vfma(y1A, ipA, m2B), dm3);          // dm3 + dm2 (m2A + m2B)
    const V dm36 = vfma(ndm1, vneg(vfma(y2, ipA, m1B)), dm3);    // dm3 + dm1 (m1A + m1B)
    const V y1irA = vmul(y1A, irA), dy1ir = vfma(dy1, irB, vneg(vmul(y1A, ndir)));
    const V y2irA = vmul(y2, irA), ndy2ir = vmul(y2, ndir);
    const V nairA = vmul(KN(K_AA), irA), ndair = vfma(KN(K_DA), irB, vmul(aA, ndir));
    const V m10B = vmul(y2, iqB), ndm10 = vmul(y2, ndiq);
    const V m11B = vmul(z1B, iqB), dm11 = vfma(dz1, iqB, vneg(vmul(z1A, ndiq)));
    const V c12 = vmul(sg, KC(K_C1M12));              // signed coefficient of the (m10 · r⁻¹) products
    // The r⁻¹-weighted monomials share two brackets (distributivity of Δ(u v) = Δu v_B + u_A Δv):
    //   v1: -b1 Δ(y1 r⁻¹ m1) + b2 Δ(y1 r⁻¹ m2) - b2 Δ(y1 r⁻¹ m11) + c12 Δ(y1 r⁻¹ m10)
    //       = Δ(y1 r⁻¹)·X1 + (y1 r⁻¹)_A·ΔX1
    //   v3: the same brackets with a r⁻¹ in place of y1 r⁻¹, negated
    //   v2: b2 Δ(y1 r⁻¹ m1) + Δ(y2 r⁻¹)·X2 + (y2 r⁻¹)_A·ΔX2
    // (ndm1, ndm10, ndy2ir: negated differences, folded into the coefficient signs)
    const V X2 = vfma(KN(K_B1), m1B, vfma(KN(K_B2), m11B, vmul(c12, m10B)));
    const V dX2 = vfma(KC(K_B1), ndm1, vfma(KN(K_B2), dm11, vneg(vmul(c12, ndm10))));
    const V X1 = vfma(KC(K_B2), m2B, X2);
    const V dX1 = vfma(KC(K_B2), dm2, dX2);
    V v1 = vmul(KC(K_C1F), dF);
    v1 = vfma(KC(K_C1P), dLp, v1);
    if constexpr (!Steep) {
        v1 = vfma(KN(K_KC1), ndm1, v1);
        v1 = vfma(KN(K_KC2), dm2, v1);
    }
    v1 = vfma(KN(K_HB2), dm35, v1);
    v1 = vfma(KC(K_HB1), dm4, v1);
    v1 = vfma(KN(K_C1M10), ndm10, v1);
    v1 = vfma(dy1ir, X1, v1);
    v1 = vfma(y1irA, dX1, v1);
    // configuration-signed terms: sg Δlog(r - z3) and sg Δm11 (sg² = 1)
    const V sgdLq = vmul(sg, dLq), sgdm11 = vmul(sg, dm11);
    if constexpr (!Steep) v1 = vfma(KC(K_C1Q), sgdLq, v1);
    v1 = vfma(KC(K_C1M11), sgdm11, v1);
    V v2 = vmul(KC(K_C2F), dF);
    v2 = vfma(KC(K_C2P), dLp, v2);
    if constexpr (!Steep) {
        v2 = vfma(KC(K_KC2), ndm1, v2);
        v2 = vfma(KN(K_KC1), dm2, v2);
    }
    v2 = vfma(KC(K_HB1), dm36, v2);
    v2 = vfma(KN(K_HB2), dm4, v2);
    v2 = vfma(KC(K_B2), vfma(dy1ir, m1B, vneg(vmul(y1irA, ndm1))), v2);
    v2 = vfma(vneg(ndy2ir), X2, v2);
    v2 = vfma(y2irA, dX2, v2);
    v2 = vfma(KC(K_C2Q), sgdLq, v2);
    V v3 = vmul(KC(K_C3F), dF);
    if constexpr (!Steep) v3 = vfma(KN(K_KC2L), dLp, v3);
    v3 = vfma(KN(K_NB1), ndm1, v3);
    v3 = vfma(KN(K_NB2), dm2, v3);
    v3 = vfma(KN(K_C3M10), ndm10, v3);
    v3 = vfma(ndair, X1, v3);
    v3 = vfma(nairA, dX1, v3);
    if constexpr (!Steep) v3 = vfma(KC(K_C3Q), sgdLq, v3);
    v3 = vfma(KC(K_C3M11), sgdm11, v3);
    if constexpr (Steep) {
        // Near-vertical side, ratio configuration (β' = β or β - π, t = tan(β'/2), |t| < 0.17).
        // The terms whose coefficients grow like cot β or cot²β form, with p = r + a, q = r - z3,
        // m1 = y2/p, m2 = y1/p, φ = atan2(y2, p cot(β'/2) - y1) and natural logarithms,
        //   v1: 2 b1 Δφ - k b1 cot β R_F + k b2 cot β R_Q,   v2: 2 b2 Δφ + k b2 cot β R_F + k b1 cot β R_Q,
        //   v3: -k b2 cot β Q,
        //   R_F = 2 cot β Δφ - Δm1,   R_Q = cot β Q - Δm2,   Q = Δlog p - |cos β| Δlog q,
        // where R_F, R_Q and Q are O(β).  Without cancellation:
        //   * φ = atan(t μ) + const with μ = y2/(p - t y1), and 2 cot β = (1 - t²)/t, so
        //     k cot β R_F = k (1 - t²)/2 · [(1 - t²) Δ(μ m2 - t μ³ A(t²μ²)) - t Δm1]
        //     with A(u) = (w - atan w)/w³ = 1/3 - u/5 + u²/7 - ... (u = w² < 0.04: three terms);
        //   * c = p - q = a (1 - |cos β|) + sg y1 sin β and E = c/q give p = q (1 + E),
        //     Q = Δlog(1 + E) + (1 - |cos β|) Δlog q and cot β E - m2 = E m2 + (1 - |cos β|)(a cot β - y1)/q,
        //     R_Q = cot β Δλ + Δ(E m2) + (1 - |cos β|) (Δ((a cot β - y1)/q) + cot β Δlog q),
        //     λ = log(1 + E) - E, Δλ = -s (E_A + E_B) + 2 s³ (1/3 + s²/5 + s⁴/7 + ...), s = ΔE/(2 + E_A + E_B);
        // every difference from (value at A, difference) pairs.  What is left has O(1) terms:
        // -k b1/2 = -hb1 and k b2/2 = hb2 on G = (1 - t²)[...], and k b2 cot β, k b1 cot β on R_Q = O(β).
        const V cot = KC(K_COT), omc = KC(K_OMC), t = KC(K_T), nt = KN(K_T);
        const V cA = vfma(KC(K_SSB), y1A, KC(K_A1C));
        const V EA = vmul(cA, iqA);
        const V dE = vfma(KC(K_DC), iqB, vneg(vmul(cA, ndiq)));
        const V EAB = vadd(vadd(EA, EA), dE);                           // E_A + E_B
        const V sE = vmul(dE, frcp(vadd(V(2.0f), EAB)));
        const V s2 = vmul(sE, sE);
        V P = vfma(s2, V(1.0f / 11.0f), V(1.0f / 9.0f));
        P = vfma(P, s2, V(1.0f / 7.0f));
        P = vfma(P, s2, V(1.0f / 5.0f));
        P = vfma(P, s2, V(1.0f / 3.0f));
        const V dlam = vfma(vmul(vadd(sE, sE), s2), P, vneg(vmul(sE, EAB)));
        const V dlnq = vmul(V(0.693147181f), dLq);
        const V uA = vfma(aA, cot, vneg(y1A));                           // a cot β - y1 at A
        const V du = vfma(da, cot, KN(K_DY1));
        const V dW = vfma(du, iqB, vneg(vmul(uA, ndiq)));
        V RQ = vfma(dE, m2B, vmul(EA, dm2));
        RQ = vfma(cot, dlam, RQ);
        RQ = vfma(omc, vfma(cot, dlnq, dW), RQ);
        const V Qn = vfma(omc, dlnq, vadd(dlam, dE));
        // μ at A and B, Δμ = -y2 (Δp - t Δy1)/(D_A D_B) with D = p - t y1 > 0
        const V iDA = frcp(vfma(nt, y1A, pA)), iDB = frcp(vfma(nt, y1B, pB));
        const V muA = vmul(y2, iDA), muB = vmul(y2, iDB);
        const V dmu = vmul(vmul(vneg(y2), vfma(nt, KC(K_DY1), dp)), vmul(iDA, iDB));
        const V dmm = vfma(dmu, m2B, vmul(muA, dm2));                   // Δ(μ m2)
        // t μ³ A(t²μ²): an O(t) correction, differenced directly
        auto cubic = [&](V mu) {
            const V w = vmul(t, mu), u = vmul(w, w);
            const V a = vfma(vfma(u, V(1.0f / 7.0f), V(-1.0f / 5.0f)), u, V(1.0f / 3.0f));
            return vmul(vmul(w, vmul(mu, mu)), a);
        };
        const V omt2 = vfma(nt, t, V(1.0f));
        const V G = vmul(omt2, vfma(omt2, vsub(dmm, vsub(cubic(muB), cubic(muA))), vmul(t, ndm1)));
        v1 = vfma(KN(K_HB1), G, v1);
        v2 = vfma(KC(K_HB2), G, v2);
        v1 = vfma(KC(K_KR1), RQ, v1);
        v2 = vfma(KC(K_KR2), RQ, v2);
        v3 = vfma(KN(K_KR1), Qn, v3);
    }
    // back to EFCS: columns e1 = (c, s, 0), e2 = (s, -c, 0), e3 = (0, 0, -1); v3 is summed on
    // its own before it meets the running total (finer rounding than adding term by term)
    ue = vfma(c, v1, vfma(s, v2, ue));
    un = vfma(s, v1, vfma(KN(K_C), v2, un));
    uv = vsub(uv, v3);
}

// One pair, with the near-vertical evaluation for steep sides (a warp-uniform choice per side)
template <class V, class K>
AG_DEVICE_INLINE void side_pair(const K& k, V Xr, V Yr, V& ue, V& un, V& uv, bool steep) {
    if (steep)
        side_pair_t<true>(k, Xr, Yr, ue, un, uv);
    else
        side_pair_t<false>(k, Xr, Yr, ue, un, uv);
}

// One rectangle by nn quadrature nodes (from rect_node; the point tensile dislocation above).
// Per station: the strike-frame coordinates and q once, then per node, with s = 1/(R(R+d)),
//   R² = x² + y² + d², A = s/(R+d) = 1/(R(R+d)²), E = A/R² = 1/(R³(R+d)²),
//   B = (3R+d) E/(R+d), T = 3q²/R⁵,
//   ux = x [T - k s² (1/R³ - (A - y² B))],  uy = y [T - k s² (A - x² B)],
//   uz = d T - k s² (s - x²(2R+d) E),
// weighted and summed in FP32 (the nodes' terms vary smoothly: no cancellation).  The node
// weight w enters as W = w (-k sin²δ), formed once per node for all of a lane's stations, and
// as w T per station, so each component's weighted term is one FMA into its sum.
template <class V>
AG_DEVICE_INLINE void rect_quad(const RectQ& Q, const float4* node, int nn, V Xr, V Yr, V& ue, V& un, V& uv) {
    const V a = V(Q.h0.x), b = V(Q.h0.y);
    const V xs = vfma(a, Xr, vmul(b, Yr));
    const V ys = vfma(a, Yr, vneg(vmul(b, Xr)));
    const V q = vfma(ys, V(Q.h0.z), V(-Q.h0.w));
    const V q3 = vmul(vmul(q, q), V(3.0f));
    V sx(0.0f), sy(0.0f), sz(0.0f);
#pragma unroll 2
    for (int k = 0; k < nn; ++k) {
        const float4 nd = node[k];
        const V x = vsub(xs, V(nd.x)), y = vsub(ys, V(nd.y)), d = V(nd.z), w = V(nd.w);
        const V W = V(__fmul_rn(nd.w, Q.h1.x));
        const V x2 = vmul(x, x), y2 = vmul(y, y);
        const V R2 = vfma(d, d, vadd(x2, y2));
        const V iR = vrsqrt(R2);
        const V R = vmul(R2, iR);
        const V iRd = frcp(vadd(R, d));
        const V s = vmul(iR, iRd);
        const V A = vmul(s, iRd);
        const V iR2 = vmul(iR, iR);
        const V E = vmul(A, iR2);
        const V iR3 = vmul(iR2, iR);
        const V Tw = vmul(vmul(q3, w), vmul(iR3, iR2));
        const V B = vmul(vmul(vfma(V(3.0f), R, d), E), iRd);
        const V G1 = vfma(vneg(x2), B, A);
        const V G2 = vfma(vneg(y2), B, A);
        const V I5 = vfma(vneg(vmul(x2, vfma(V(2.0f), R, d))), E, s);
        sx = vfma(x, vfma(W, vsub(iR3, G2), Tw), sx);
        sy = vfma(y, vfma(W, G1, Tw), sy);
        sz = vfma(W, I5, vfma(d, Tw, sz));
    }
    // back to EFCS: x̂ = (a, b), ŷ = (-b, a)
    ue = vfma(a, sx, vfma(vneg(b), sy, ue));
    un = vfma(b, sx, vfma(a, sy, un));
    uv = vadd(uv, sz);
}

#undef KC
#undef KN

}  // namespace ag
