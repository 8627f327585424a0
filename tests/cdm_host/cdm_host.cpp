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
#include <algorithm>
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

// Bounding boxes of the tiles of kTileSize consecutive stations, as the library forms them
// (coordinates split into FP32 hi + lo, the box rounded outwards)
static const int kTileSize = 128;
static void tile_boxes(const double* X, const double* Y, int n, float* box) {
    for (int t = 0; t * kTileSize < n; ++t) {
        double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
        for (int j = t * kTileSize; j < n && j < (t + 1) * kTileSize; ++j) {
            float ah, al, bh, bl;
            split_hilo(X[j], ah, al);
            split_hilo(Y[j], bh, bl);
            const double x = (double)ah + (double)al, y = (double)bh + (double)bl;
            x0 = std::fmin(x0, x); x1 = std::fmax(x1, x);
            y0 = std::fmin(y0, y); y1 = std::fmax(y1, y);
        }
        box[4 * t] = f32_down(x0); box[4 * t + 1] = f32_up(x1);
        box[4 * t + 2] = f32_down(y0); box[4 * t + 3] = f32_up(y1);
    }
}

// LOS displacements of one source at n stations, evaluated as the likelihood kernel does:
// stations in tiles of kTileSize in the given order, each tile with its own plan
extern "C" int cdm_host_los(const double* th, int n, const double* X, const double* Y, const double* los,
                            double nu, double* out) {
    HostLayout L{0, 2, 3, 4, 7, nu};
    Vec3 V[3][4];
    if (cdm_corners(th, L, V)) return -1;
    SideC side[kSides];
    RectQ rect[3];
    const double x0 = th[0], y0 = th[1];
    const uint32_t mask = cdm_sides(th, L, V, x0, y0, side, rect);
    float x0h, x0l, y0h, y0l;
    split_hilo(x0, x0h, x0l);
    split_hilo(y0, y0h, y0l);
    const int ntiles = (n + kTileSize - 1) / kTileSize;
    float* box = new float[4 * ntiles];
    tile_boxes(X, Y, n, box);
    float4 node[kQuadBudget];
    for (int t = 0; t < ntiles; ++t) {
        const float* tb = box + 4 * t;
        const float bx0 = (tb[0] - x0h) - x0l, bx1 = (tb[1] - x0h) - x0l;
        const float by0 = (tb[2] - y0h) - y0l, by1 = (tb[3] - y0h) - y0l;
        uint32_t sides = mask & 0x0FFFu, qrect = 0u;
        int qn[3][2] = {};
        for (int r = 0; r < 3; ++r)
            if ((mask >> (27 + r) & 1u) &&
                tile_quad(rect[r], (mask >> (24 + r)) & 1u, bx0, bx1, by0, by1, qn[r][0], qn[r][1])) {
                qrect |= 1u << r;
                sides &= ~(0xFu << (4 * r));
            }
        for (int j = t * kTileSize; j < n && j < (t + 1) * kTileSize; ++j) {
            float ah, al, bh, bl;
            split_hilo(X[j], ah, al);
            split_hilo(Y[j], bh, bl);
            const float Xr = (ah - x0h) + (al - x0l), Yr = (bh - y0h) + (bl - y0l);
            float ue = 0.f, un = 0.f, uv = 0.f;
            for (int k = 0; k < kSides; ++k)
                if (sides >> k & 1u)
                    side_pair<float>(ScalarSide(side[k]), Xr, Yr, ue, un, uv, (mask >> (kSides + k)) & 1u);
            for (int r = 0; r < 3; ++r) {
                if (!(qrect >> r & 1u)) continue;
                const int nn = qn[r][0] * qn[r][1];
                for (int k = 0; k < nn; ++k) node[k] = rect_node(rect[r], qn[r][0], qn[r][1], k, kGaussXf, kGaussWf);
                rect_quad<float>(rect[r], node, nn, Xr, Yr, ue, un, uv);
            }
            out[j] = (double)ue * los[3 * j] + (double)un * los[3 * j + 1] + (double)uv * los[3 * j + 2];
        }
    }
    delete[] box;
    return 0;
}

// plan of one source (mask: sides, steep sides, far rectangles, rectangles taking part; far
// node counts) and the work of the likelihood kernel over m stations in the given tiles
// (boxes as from ag_station_boxes), summed as ag_cdm_work sums it
extern "C" int cdm_host_plan(const double* th, double nu, const float* box, int m, uint32_t* mask, int* nq,
                             double* flop, double* sfu) {
    HostLayout L{0, 2, 3, 4, 7, nu};
    Vec3 V[3][4];
    if (cdm_corners(th, L, V)) return -1;
    int q[3][2];
    *mask = cdm_plan(th, L, V, q);
    for (int r = 0; r < 3; ++r) nq[2 * r] = q[r][0], nq[2 * r + 1] = q[r][1];
    RectQ rect[3];
    cdm_rects(th, L, V, th[0], th[1], rect);
    float x0h, x0l, y0h, y0l;
    split_hilo(th[0], x0h, x0l);
    split_hilo(th[1], y0h, y0l);
    double f = 0.0, u = 0.0;
    for (int t = 0; t * kTileSize < m; ++t) {
        const float* tb = box + 4 * t;
        uint32_t fl, su;
        tile_work(rect, *mask, (tb[0] - x0h) - x0l, (tb[1] - x0h) - x0l, (tb[2] - y0h) - y0l, (tb[3] - y0h) - y0l,
                  fl, su);
        const int cnt = std::min(kTileSize, m - t * kTileSize);
        f += (double)fl * cnt;
        u += (double)su * cnt;
    }
    *flop = f;
    *sfu = u;
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
        RectQ R;
        fill_rect(R, P, 2.0, 0.25, 0, 0, 0, nn, 1);
        float4 node[2];
        for (int k = 0; k < nn; ++k) node[k] = rect_node(R, nn, 1, k, kGaussXf, kGaussWf);
        CountF ue(0.f), un(0.f), uv(0.f);
        g_flop = g_sfu = 0;
        rect_quad<CountF>(R, node, nn, CountF(1000.f), CountF(-2000.f), ue, un, uv);
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
