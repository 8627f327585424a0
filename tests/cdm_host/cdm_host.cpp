// Host build of the CDM per-side arithmetic of the likelihood kernel (test harness).
//
// The device header altar_gb300/csrc/cdm_side.cuh is compiled here with g++ so that
// its formulas can be checked on a machine without a GPU:
//   * cdm_host_los: displacements of one source at a set of stations, with the device
//     intrinsics replaced by correctly rounded host operations (the kernel's approximate
//     reciprocal, reciprocal square root and base-2 logarithm differ from these by a
//     few ulp), to compare against the FP64 oracle;
//   * cdm_host_side_counts / cdm_host_quad_counts: the static operation counts of one side
//     and of one quadrature node (FP32 FLOP with an FMA counted as 2, and special-function
//     operations), by evaluating them with a counting number type;
//   * cdm_host_plan: the per-chain plan (sides or quadrature per rectangle) and its work.
#include <cmath>
#include <cstdint>

#define __host__
#define __device__
#define __forceinline__ inline
#define __align__(n) alignas(n)
struct float4 { float x, y, z, w; };
static inline float4 make_float4(float a, float b, float c, float d) { return {a, b, c, d}; }
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __fmul_rn(float a, float b) { return a * b; }
static inline float __fdividef(float a, float b) { return a / b; }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
#define __log2f(x) std::log2(x)
#include <cstring>
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline int __float_as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
#define AG_GL_TABLE static const
static inline void sincospi(double x, double* s, double* c) {
    *s = std::sin(M_PI * x);
    *c = std::cos(M_PI * x);
}
#define AG_DEVICE_INLINE inline
#define AG_CDM_FN inline
#include "../../altar_gb300/csrc/cdm_side.cuh"

using namespace ag;

// parameter positions of the CDM workload layout: x, y, depth, opening, ax, ay, az, ωx, ωy, ωz
struct HostLayout { int x_idx, depth_idx, strength_idx, axes_idx, omega_idx; double nu; };

extern "C" int cdm_host_los(const double* th, int n, const double* X, const double* Y, const double* los,
                            double nu, double* out) {
    HostLayout L{0, 2, 3, 4, 7, nu};
    Vec3 V[3][4];
    if (cdm_corners(th, L, V)) return -1;
    SideC side[kSides];
    const double x0 = th[0], y0 = th[1];
    const uint32_t mask = cdm_sides(th, L, V, x0, y0, side);
    float x0h, x0l, y0h, y0l;
    split_hilo(x0, x0h, x0l);
    split_hilo(y0, y0h, y0l);
    for (int j = 0; j < n; ++j) {
        float ah, al, bh, bl;
        split_hilo(X[j], ah, al);
        split_hilo(Y[j], bh, bl);
        const float Xr = (ah - x0h) + (al - x0l), Yr = (bh - y0h) + (bl - y0l);
        float ue = 0.f, un = 0.f, uv = 0.f;
        for (int k = 0; k < kSides; ++k)
            if (mask >> k & 1u) side_pair<float>(ScalarSide(side[k]), Xr, Yr, ue, un, uv, (mask >> (kSides + k)) & 1u);
        for (int r = 0; r < 3; ++r)
            if (mask >> (24 + r) & 1u) rect_quad<float>(*reinterpret_cast<const QuadC*>(&side[4 * r]), Xr, Yr, ue, un, uv);
        out[j] = (double)ue * los[3 * j] + (double)un * los[3 * j + 1] + (double)uv * los[3 * j + 2];
    }
    return 0;
}

// plan of one source: mask (sides, steep sides, quadrature rectangles) and node counts
extern "C" int cdm_host_plan(const double* th, double nu, uint32_t* mask, int* nq, uint32_t* flop, uint32_t* sfu) {
    HostLayout L{0, 2, 3, 4, 7, nu};
    Vec3 V[3][4];
    if (cdm_corners(th, L, V)) return -1;
    int q[3][2];
    *mask = cdm_plan(th, L, V, q);
    for (int r = 0; r < 3; ++r) nq[2 * r] = q[r][0], nq[2 * r + 1] = q[r][1];
    cdm_work(*mask, q, *flop, *sfu);
    return 0;
}

// the library's work constants, for comparison with the counted figures
extern "C" void cdm_host_work_constants(int* out) {
    out[0] = kFlopSide; out[1] = kFlopSteepExtra; out[2] = kFlopQuadRect; out[3] = kFlopQuadNode;
    out[4] = kFlopStation; out[5] = kSfuSide; out[6] = kSfuSteepExtra; out[7] = kSfuQuadNode;
}

// ---------------------------------------------------------------------------
// operation counting
static long g_flop = 0, g_sfu = 0;
struct CountF { float v; CountF() {} CountF(float x) : v(x) {} };
struct CountB { bool v; };
inline CountF vfma(CountF a, CountF b, CountF c) { g_flop += 2; return std::fma(a.v, b.v, c.v); }
inline CountF vadd(CountF a, CountF b) { g_flop += 1; return a.v + b.v; }
inline CountF vsub(CountF a, CountF b) { g_flop += 1; return a.v - b.v; }
inline CountF vmul(CountF a, CountF b) { g_flop += 1; return a.v * b.v; }
inline CountF vneg(CountF a) { return -a.v; }
inline CountB vge0(CountF a) { return {a.v >= 0.f}; }
inline CountB vgt0(CountF a) { return {a.v > 0.f}; }
inline CountB vand(CountB a, CountB b) { return {a.v && b.v}; }
inline CountF vsel(CountB c, CountF a, CountF b) { return c.v ? a : b; }
inline CountF frcp(CountF x) { g_sfu += 1; return 1.0f / x.v; }
inline CountF vrsqrt(CountF x) { g_sfu += 1; return 1.0f / std::sqrt(x.v); }
// log2_ratio: s², 4 FMA, s·p (10 FLOP) + one base-2 logarithm
inline CountF vlog2r(CountF s, CountF r) { g_flop += 10; g_sfu += 1; return log2_ratio(s.v, r.v); }
// atan2_poly: mx + 1e-30, mn/mx (mul), t², 8 FMA, t·p, two quadrant subtractions (22 FLOP)
// + one reciprocal
inline CountF vatan2(CountF y, CountF x) { g_flop += 22; g_sfu += 1; return atan2_poly(y.v, x.v); }

// quadrature: FLOP and special-function operations of a rectangle with one node and with two
extern "C" void cdm_host_quad_counts(long* flop1, long* sfu1, long* flop2, long* sfu2) {
    const Vec3 P[4] = {{-500, 300, -4000}, {700, 200, -3500}, {650, 900, -3300}, {-550, 1000, -3800}};
    for (int nn = 1; nn <= 2; ++nn) {
        QuadC Q;
        fill_quad(Q, P, 2.0, 0.25, 0, 0, nn, 1);
        CountF ue(0.f), un(0.f), uv(0.f);
        g_flop = g_sfu = 0;
        rect_quad<CountF>(Q, CountF(1000.f), CountF(-2000.f), ue, un, uv);
        *(nn == 1 ? flop1 : flop2) = g_flop;
        *(nn == 1 ? sfu1 : sfu2) = g_sfu;
    }
}

extern "C" void cdm_host_side_counts(long* flop, long* sfu, long* flop_steep, long* sfu_steep) {
    SideC S;
    fill_side(S, Vec3{100, 200, -3000}, Vec3{900, -300, -2500}, Vec3{1, 2, 3}, 0.25, 0, 0, false);
    for (int s = 0; s < 2; ++s) {
        CountF ue(0.f), un(0.f), uv(0.f);
        g_flop = g_sfu = 0;
        side_pair<CountF>(ScalarSide(S), CountF(1000.f), CountF(-2000.f), ue, un, uv, s == 1);
        *(s ? flop_steep : flop) = g_flop;
        *(s ? sfu_steep : sfu) = g_sfu;
    }
}
