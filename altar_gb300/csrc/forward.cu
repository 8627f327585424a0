// Fused batched forward models + diagonal-Cd misfit + per-chain log-likelihood.
//
// CDM (Compound Dislocation Model, Nikkhoo et al. 2016), following the
// reference numpy CDM models/cdm/cdm/libcdm.py:39-430, and the Mogi point
// source, following models/mogi/lib/libmogi/Source.cc:65-154.
//
// CDM evaluation strategy.  The reference sums, over the 12 sides of three
// rectangles, the difference v(B) - v(A) of two angular dislocations
// (libcdm.py:310-372).  Evaluated in FP32 as written, that difference loses
// up to ~4 digits: each term is O(1) while the side's contribution is
// O(side length / distance).  Here every quantity of the angular-dislocation
// formula is carried as a pair (value at A, difference B - A), with the
// difference propagated by exact identities (product rule
// Δ(uv) = Δu·v_B + u_A·Δv, Δ(1/u) = -Δu/(u_A u_B),
// Δr = Δ(r²)/(r_A + r_B), Δlog u = log1p(Δu/u_A), and the Burgers-function
// difference as a single atan2 of the rotation from A to B), so the
// cancellation never happens in floating point.
//
// Work decomposition: cdm_setup_kernel computes each chain's per-side
// constants in FP64 and packs the chains that have work (not masked, not
// above the free surface) into consecutive slots; the likelihood kernel runs
// one warp per slot, lanes over stations; a CTA holds WARPS chains whose
// constants live in shared memory and are read with broadcast vector loads;
// station tiles stream through a ring of shared-memory buffers filled by 1-D
// bulk copies (cp.async.bulk + mbarrier) and shared by the CTA's warps.  Each
// lane accumulates w·r² in float-float; the warp's sum is reduced in FP64 in
// a fixed order.
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"

namespace ag {

constexpr int kMaxOffsets = 16;      // datasets with their own offset parameter
constexpr int kSides = 12;
constexpr int kTile = AG_STATION_TILE;
constexpr uint32_t kWaitLimit = 1u << 24;

// ---------------------------------------------------------------------------
// per-side constants of one angular-dislocation pair (36 floats)
struct __align__(16) SideC {
    float4 q[9];
};
// q0: c, s, k1, k2          frame (unit horizontal side direction) and vertex A
// q1: dy1, aA, aB, da       y1(B) - y1(A); depths of A and B; aB - aA
// q2: sb, cb, tb2, ctb2     sin β, cos β, tan(β/2), cot(β/2) (configuration II)
// q3: daS, C1F, C2F, C3F    da·(aA+aB); coefficients of ΔFi
// q4: C1P, C2P, kc1, kc2    coefficients of Δlog(r+a); k·cot·b1, k·cot·b2
// q5: nb1, nb2, hb1, hb2    2ν b1, 2ν b2, k b1/2, k b2/2
// q6: b1, b2, C1m10, C3m10
// q7: C1Q, C2Q, C3Q, C1m11  configuration-signed coefficients
// q8: C3m11, C1m12, 0, 0

struct __align__(16) ChainC {
    float4 hdr;                 // x0_hi, x0_lo, y0_hi, y0_lo
    uint32_t side_mask;         // active sides; 0 = chain inactive
    uint32_t status;
    uint32_t pad0, pad1;
    float off[kMaxOffsets];     // per-dataset offsets θ[offset_idx + k]
    float pad2[8];
    SideC side[kSides];
};
static_assert(sizeof(ChainC) % 16 == 0, "ChainC must be a whole number of float4");

// ---------------------------------------------------------------------------
// FP64 per-chain set-up: rotation, corners, geometry check, per-side constants
struct Vec3 { double x, y, z; };
__device__ inline Vec3 v_sub(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline Vec3 v_add(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline Vec3 v_scale(Vec3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline Vec3 v_cross(Vec3 a, Vec3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ inline double v_dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ inline void split_hilo(double v, float& hi, float& lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

__device__ void fill_side(SideC& S, Vec3 pa, Vec3 pb, Vec3 bvec, double nu, double x0, double y0,
                          bool& active) {
    const double PI = 3.14159265358979323846;
    Vec3 side = v_sub(pb, pa);
    double L = sqrt(v_dot(side, side));
    double beta = acos(-side.z / L);
    // vertical sides contribute nothing (libcdm.py:320-324)
    const double eps = 2.220446049250313e-16;
    if (!(L > 0.0) || fabs(beta) < eps || fabs(PI - beta) < eps) {
        active = false;
        return;
    }
    active = true;
    double hl = sqrt(side.x * side.x + side.y * side.y);
    double c = side.x / hl, s = side.y / hl;         // e1 = (c, s, 0), e2 = (s, -c, 0)
    double sb = hl / L, cb = -side.z / L;            // β in (0, π): sin β >= 0
    double tb2 = (cb >= 0.0) ? sb / (1.0 + cb) : (1.0 - cb) / sb;
    double ctb2 = 1.0 / tb2;
    double cot = cb / sb;
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
    double C2Q = -kc1 / sb;
    double C3Q = kc2 * cb;
    double C1m11 = b2 * sb;
    double C3m11 = b2 * cb;
    double C1m12 = b1 * cb - b3 * sb;
    S.q[0] = make_float4((float)c, (float)s, (float)k1, (float)k2);
    S.q[1] = make_float4((float)dy1, (float)aA, (float)aB, (float)da);
    S.q[2] = make_float4((float)sb, (float)cb, (float)tb2, (float)ctb2);
    S.q[3] = make_float4((float)(da * (aA + aB)), (float)C1F, (float)C2F, (float)C3F);
    S.q[4] = make_float4((float)C1P, (float)C2P, (float)kc1, (float)kc2);
    S.q[5] = make_float4((float)(2.0 * nu * b1), (float)(2.0 * nu * b2), (float)(0.5 * k * b1),
                         (float)(0.5 * k * b2));
    S.q[6] = make_float4((float)b1, (float)b2, (float)C1m10, (float)C3m10);
    S.q[7] = make_float4((float)C1Q, (float)C2Q, (float)C3Q, (float)C1m11);
    S.q[8] = make_float4((float)C3m11, (float)C1m12, 0.f, 0.f);
}

// corners of the three rectangles (libcdm.py:174-217); returns true if any is above the surface
__device__ bool cdm_corners(const double* th, const ag_layout& L, Vec3 V[3][4]) {
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

// One thread per requested chain (all n, or the first *count_in of index_in).  Chains that
// are masked or lie above the free surface get their status and nothing else; every other
// chain takes the next compacted slot (slot order is the order of the atomic, which does not
// affect any chain's result) and writes its constants there, so the likelihood kernel's CTAs
// hold only chains with work.
__global__ void cdm_setup_kernel(ag_layout L, const double* __restrict__ theta, int n,
                                 const uint32_t* __restrict__ mask_in, ChainC* __restrict__ out,
                                 uint32_t* __restrict__ chain_status, int noffsets,
                                 const int32_t* __restrict__ index_in, const int32_t* __restrict__ count_in,
                                 int32_t* __restrict__ index_out, int32_t* __restrict__ count_out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i = t;
    if (index_in) {
        if (t >= *count_in) return;
        i = index_in[t];
    }
    if (mask_in && mask_in[i]) return;
    const double* th = theta + (size_t)i * L.nparams;
    Vec3 V[3][4];
    const bool above = cdm_corners(th, L, V);
    if (above) {
        if (chain_status) chain_status[i] |= CHAIN_ABOVE_SURFACE;
        return;
    }
    const int slot = atomicAdd(count_out, 1);
    index_out[slot] = i;
    ChainC& C = out[slot];
    C.side_mask = 0u;
    C.status = 0u;
    const double x0 = th[L.x_idx], y0 = th[L.x_idx + 1];
    split_hilo(x0, C.hdr.x, C.hdr.y);
    split_hilo(y0, C.hdr.z, C.hdr.w);
    for (int k = 0; k < kMaxOffsets; ++k)
        C.off[k] = (k < noffsets) ? (float)th[L.offset_idx + k] : 0.f;
    // which rectangles take part (libcdm.py:226-242)
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
    const double opening = th[L.strength_idx];
    uint32_t mask = 0u;
    for (int r = 0; r < 3; ++r) {
        if (!use[r]) continue;
        Vec3 nrm = v_cross(v_sub(V[r][1], V[r][0]), v_sub(V[r][3], V[r][0]));
        nrm = v_scale(nrm, 1.0 / sqrt(v_dot(nrm, nrm)));
        Vec3 b = v_scale(nrm, opening);
        for (int e = 0; e < 4; ++e) {
            bool act;
            fill_side(C.side[r * 4 + e], V[r][e], V[r][(e + 1) & 3], b, L.nu, x0, y0, act);
            if (act) mask |= 1u << (r * 4 + e);
        }
    }
    // a chain with no active side still needs a llk: keep bit 31 as "evaluate"
    C.side_mask = mask | 0x80000000u;
}

__global__ void cdm_check_kernel(ag_layout L, const double* __restrict__ theta, int n,
                                 uint32_t* __restrict__ chain_status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Vec3 V[3][4];
    if (cdm_corners(theta + (size_t)i * L.nparams, L, V)) chain_status[i] |= CHAIN_ABOVE_SURFACE;
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
AG_DEVICE_INLINE float vlog1p(float x) { return log1p_series(x); }
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
template <int N> AG_DEVICE_INLINE SV<N> vlog1p(SV<N> x) { AG_SV_MAP(log1p_series(x.v[i])); }
template <int N> AG_DEVICE_INLINE SV<N> vatan2(SV<N> y, SV<N> x) { AG_SV_MAP(atan2_poly(y.v[i], x.v[i])); }
#undef AG_SV_MAP
#undef AG_CV_MAP

// Per-side constant by its position in SideC (q[i >> 2], component i & 3)
enum : int {
    K_C = 0, K_S, K_K1, K_K2, K_DY1, K_AA, K_AB, K_DA, K_SB, K_CB, K_TB2, K_CTB2, K_DAS, K_C1F, K_C2F, K_C3F,
    K_C1P, K_C2P, K_KC1, K_KC2, K_NB1, K_NB2, K_HB1, K_HB2, K_B1, K_B2, K_C1M10, K_C3M10, K_C1Q, K_C2Q, K_C3Q,
    K_C1M11, K_C3M11, K_C1M12
};

struct ScalarSide {
    float4 q[9];
    AG_DEVICE_INLINE explicit ScalarSide(const SideC& S) {
#pragma unroll
        for (int i = 0; i < 9; ++i) q[i] = S.q[i];
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
// one angular-dislocation pair in difference arithmetic
template <class V, class K>
AG_DEVICE_INLINE void side_pair(const K& k, V Xr, V Yr, V& ue, V& un, V& uv) {
    const V c = KC(K_C), s = KC(K_S);
    const V dy1 = KC(K_DY1), aA = KC(K_AA), aB = KC(K_AB), da = KC(K_DA);
    // station in the angular-dislocation frame of vertex A; y2 is the same at B
    const V y1A = vfma(c, Xr, vfma(s, Yr, KN(K_K1)));
    const V y2 = vfma(s, Xr, vfma(KN(K_C), Yr, KN(K_K2)));
    const V y1B = vadd(y1A, dy1);
    // artefact-free configuration (libcdm.py:342-362): I if y1A >= 0 (β - π), else II (β)
    const auto conf1 = vge0(y1A);
    const V sg = vsel(conf1, V(-1.0f), V(1.0f));
    const V sB = vmul(sg, KC(K_SB)), cB = vmul(sg, KC(K_CB)), ncB = vmul(sg, KN(K_CB));
    const V ct2 = vsel(conf1, KN(K_TB2), KC(K_CTB2));
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
    // z1, z3
    const V z1A = vfma(y1A, cB, vmul(aA, sB));
    const V dz1 = vfma(dy1, cB, vmul(da, sB));
    const V z1B = vadd(z1A, dz1);
    const V z3A = vfma(y1A, sB, vmul(aA, ncB));
    const V dz3 = vfma(dy1, sB, vmul(da, ncB));
    const V z3B = vadd(z3A, dz3);
    // r - z3, cancellation-free: (z1² + y2²)/(r + z3) when z3 > 0, else (r + z3) - 2 z3
    const auto posA = vgt0(z3A), posB = vgt0(z3B);
    const V NA = vfma(z1A, z1A, y22), NB = vfma(z1B, z1B, y22);
    const V DA = vfma(r2A, irA, z3A), DB = vfma(r2B, irB, z3B);
    const V uA = vsel(posA, NA, vfma(V(-2.0f), z3A, DA)), vA = vsel(posA, DA, V(1.0f));
    const V uB = vsel(posB, NB, vfma(V(-2.0f), z3B, DB)), vB = vsel(posB, DB, V(1.0f));
    const V iuA = frcp(uA), ivA = frcp(vA), iuB = frcp(uB), ivB = frcp(vB);
    const V iqA = vmul(vA, iuA), iqB = vmul(vB, iuB);
    const V dN = vmul(dz1, vadd(z1A, z1B));
    const V dq = vsel(vand(posA, posB), vmul(vmul(vfma(dN, DA, vneg(vmul(NA, vadd(dr, dz3)))), ivA), ivB),
                      vsub(dr, dz3));
    const V ndiq = vmul(vmul(dq, iqA), iqB);           // -Δ(1/q)
    // log differences
    const V dLp = vlog1p(vmul(dp, ipA));
    const V dLq = vlog1p(vmul(dq, iqA));
    // Burgers function difference: rotation of (x, y2) from A to B; y2 keeps its sign so
    // the rotation never crosses atan2's cut
    const V xA = vfma(pA, ct2, vneg(y1A));
    const V dx = vfma(dp, ct2, KN(K_DY1));
    const V xB = vadd(xA, dx);
    const V dF = vmul(V(2.0f), vatan2(vmul(vneg(y2), dx), vfma(xA, xB, y22)));
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
    v1 = vfma(KN(K_KC1), ndm1, v1);
    v1 = vfma(KN(K_KC2), dm2, v1);
    v1 = vfma(KN(K_HB2), dm35, v1);
    v1 = vfma(KC(K_HB1), dm4, v1);
    v1 = vfma(KN(K_C1M10), ndm10, v1);
    v1 = vfma(dy1ir, X1, v1);
    v1 = vfma(y1irA, dX1, v1);
    v1 = vfma(sg, vfma(KC(K_C1Q), dLq, vmul(KC(K_C1M11), dm11)), v1);
    V v2 = vmul(KC(K_C2F), dF);
    v2 = vfma(KC(K_C2P), dLp, v2);
    v2 = vfma(KC(K_KC2), ndm1, v2);
    v2 = vfma(KN(K_KC1), dm2, v2);
    v2 = vfma(KC(K_HB1), dm36, v2);
    v2 = vfma(KN(K_HB2), dm4, v2);
    v2 = vfma(KC(K_B2), vfma(dy1ir, m1B, vneg(vmul(y1irA, ndm1))), v2);
    v2 = vfma(vneg(ndy2ir), X2, v2);
    v2 = vfma(y2irA, dX2, v2);
    v2 = vfma(vmul(sg, KC(K_C2Q)), dLq, v2);
    V v3 = vmul(KC(K_C3F), dF);
    v3 = vfma(KN(K_KC2), dLp, v3);
    v3 = vfma(KN(K_NB1), ndm1, v3);
    v3 = vfma(KN(K_NB2), dm2, v3);
    v3 = vfma(KN(K_C3M10), ndm10, v3);
    v3 = vfma(ndair, X1, v3);
    v3 = vfma(nairA, dX1, v3);
    v3 = vfma(sg, vfma(KC(K_C3Q), dLq, vmul(KC(K_C3M11), dm11)), v3);
    // back to EFCS: columns e1 = (c, s, 0), e2 = (s, -c, 0), e3 = (0, 0, -1)
    ue = vfma(c, v1, vfma(s, v2, ue));
    un = vfma(s, v1, vfma(KN(K_C), v2, un));
    uv = vsub(uv, v3);
}

#undef KC
#undef KN

// ---------------------------------------------------------------------------
// CDM likelihood.  One warp per compacted chain slot, lanes over stations.
// Station tiles stream through a ring of kStages shared-memory buffers filled
// by 1-D bulk copies: each warp waits on the buffer's full barrier, works
// through the tile and counts itself done; the warp that finishes a tile last
// refills that buffer with the tile kStages ahead.  No CTA-wide barrier is
// taken per tile, so warps drift apart by up to kStages - 1 tiles instead of
// waiting for the slowest one at every tile.
constexpr int kStages = 4;

template <int WARPS, int MINB, int SPL>
__global__ void __launch_bounds__(WARPS * 32, MINB)
cdm_llk_kernel(const ChainC* __restrict__ chains, const int32_t* __restrict__ slot_chain,
               const int32_t* __restrict__ nslots_ptr, int n, const float4* __restrict__ xy,
               const float4* __restrict__ losd, const float* __restrict__ wt,
               const int32_t* __restrict__ oid, int m, int m_padded, double norm,
               double* __restrict__ llk, float* __restrict__ resid, uint32_t* __restrict__ flags) {
    const int nslots = min(n, *nslots_ptr);
    if ((int)(blockIdx.x * WARPS) >= nslots) return;       // whole CTA past the active chains
    __shared__ ChainC s_chain[WARPS];
    __shared__ float4 s_xy[kStages][kTile];
    __shared__ float4 s_ld[kStages][kTile];
    __shared__ __align__(16) float s_w[kStages][kTile];
    __shared__ __align__(16) int32_t s_oid[kStages][kTile];
    __shared__ __align__(8) uint64_t full[kStages];
    __shared__ int s_done[kStages];
    __shared__ int s_issued;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = blockIdx.x * WARPS + warp;
    const bool active = slot < nslots;
    const int chain = active ? slot_chain[slot] : n;
    const int ntiles = m_padded / kTile;
    const bool with_oid = (oid != nullptr);
    const uint32_t tile_bytes = kTile * (16u + 16u + 4u) + (with_oid ? kTile * 4u : 0u);

    // this warp's chain constants
    if (active) {
        const float4* src = reinterpret_cast<const float4*>(chains + slot);
        float4* dst = reinterpret_cast<float4*>(&s_chain[warp]);
        constexpr int nvec = sizeof(ChainC) / 16;
        for (int k = lane; k < nvec; k += 32) dst[k] = src[k];
    }
    auto issue = [&](int t, int buf) {
        const size_t base = (size_t)t * kTile;
        mbar_arrive_expect_tx(&full[buf], tile_bytes);
        bulk_g2s(&s_xy[buf][0], xy + base, kTile * 16u, &full[buf]);
        bulk_g2s(&s_ld[buf][0], losd + base, kTile * 16u, &full[buf]);
        bulk_g2s(&s_w[buf][0], wt + base, kTile * 4u, &full[buf]);
        if (with_oid) bulk_g2s(&s_oid[buf][0], oid + base, kTile * 4u, &full[buf]);
    };
    if (threadIdx.x == 0) {
        for (int b = 0; b < kStages; ++b) {
            mbar_init(&full[b], 1);
            s_done[b] = 0;
        }
        fence_mbar_init();
        const int first = ntiles < kStages ? ntiles : kStages;
        for (int t = 0; t < first; ++t) issue(t, t);
        s_issued = first;
    }
    __syncthreads();
    const ChainC& C = s_chain[warp];
    const uint32_t smask = active ? C.side_mask : 0u;
    const float x0h = C.hdr.x, x0l = C.hdr.y, y0h = C.hdr.z, y0l = C.hdr.w;
    ff acc{0.f, 0.f};
    bool failed = false;
    for (int t = 0; t < ntiles; ++t) {
        const int buf = t % kStages;
        const uint32_t phase = (uint32_t)(t / kStages) & 1u;
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[buf], phase, kWaitLimit));
        if (!ok) {
            failed = true;
            break;
        }
        if (smask) {
            // u projected on the LOS, minus data and offset; accumulate w r² and store r
            auto finish = [&](float e_, float n_, float v_, int j) {
                const float4 B = s_ld[buf][j];
                const float w = s_w[buf][j];
                const float u = fmaf(e_, B.x, fmaf(n_, B.y, v_ * B.z));
                float r = u - B.w;
                if (with_oid) r -= C.off[s_oid[buf][j] & (kMaxOffsets - 1)];
                if (w != 0.f) ff_add_wsq(acc, r, w);
                if (resid) {
                    const int col = t * kTile + j;
                    resid[(size_t)chain * m_padded + col] = (col < m) ? r : 0.f;
                }
            };
            if constexpr (SPL > 1) {
                // stations j, j + 32, ... together; accumulation order as in the one-station loop
                for (int j0 = lane; j0 < kTile; j0 += 32 * SPL) {
                    SV<SPL> Xr, Yr;
#pragma unroll
                    for (int q = 0; q < SPL; ++q) {
                        const float4 A = s_xy[buf][j0 + 32 * q];
                        Xr.v[q] = (A.x - x0h) + (A.y - x0l);
                        Yr.v[q] = (A.z - y0h) + (A.w - y0l);
                    }
                    SV<SPL> ue(0.f), un(0.f), uv(0.f);
                    uint32_t msk = smask & 0x0FFFu;
#pragma unroll 1
                    while (msk) {
                        const int sidx = __ffs(msk) - 1;
                        msk &= msk - 1;
                        side_pair<SV<SPL>>(ScalarSide(C.side[sidx]), Xr, Yr, ue, un, uv);
                    }
#pragma unroll
                    for (int q = 0; q < SPL; ++q) finish(ue.v[q], un.v[q], uv.v[q], j0 + 32 * q);
                }
            } else {
                for (int j = lane; j < kTile; j += 32) {
                    const float4 A = s_xy[buf][j];
                    const float Xr = (A.x - x0h) + (A.y - x0l);
                    const float Yr = (A.z - y0h) + (A.w - y0l);
                    float ue = 0.f, un = 0.f, uv = 0.f;
                    uint32_t msk = smask & 0x0FFFu;
#pragma unroll 1
                    while (msk) {
                        const int sidx = __ffs(msk) - 1;
                        msk &= msk - 1;
                        side_pair<float>(ScalarSide(C.side[sidx]), Xr, Yr, ue, un, uv);
                    }
                    finish(ue, un, uv, j);
                }
            }
        }
        // done with this buffer: the last warp of the CTA to get here refills it
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            if (atomicAdd(&s_done[buf], 1) == WARPS - 1) {
                __threadfence_block();
                s_done[buf] = 0;
                if (t + kStages < ntiles) {
                    fence_proxy_async_smem();
                    issue(t + kStages, buf);
                    atomicAdd(&s_issued, 1);
                }
            }
        }
    }
    if (__syncthreads_or(failed)) {
        // a wait gave up: drain the copies still in flight (bounded) before the CTA exits
        if (threadIdx.x == 0) {
            raise_flag(flags, DEV_ERR_TIMEOUT);
            const int last = s_issued;
            for (int t = (last > kStages ? last - kStages : 0); t < last; ++t)
                mbar_wait_bounded(&full[t % kStages], (uint32_t)(t / kStages) & 1u, kWaitLimit);
        }
        return;
    }
    const double sum = warp_sum(ff_to_double(acc));
    if (lane == 0 && active) llk[chain] = norm - 0.5 * sum;
}

// ---------------------------------------------------------------------------
// Mogi: one thread per station, CH chains per CTA held in shared memory
struct __align__(16) MogiSrc {
    float4 pos;    // x0_hi, x0_lo, y0_hi, y0_lo
    float4 prm;    // depth, C = (nu - 1) ΔV / π, 0, 0
};

template <int CH, int NSRC>
__global__ void __launch_bounds__(256, 2)
mogi_llk_kernel(ag_layout L, const double* __restrict__ theta, int n,
                const uint32_t* __restrict__ mask_in, const float4* __restrict__ xy,
                const float4* __restrict__ losd, const float* __restrict__ wt,
                const int32_t* __restrict__ oid, int noffsets, int m, int m_padded, double norm,
                double* __restrict__ llk, float* __restrict__ resid, const int32_t* __restrict__ index,
                const int32_t* __restrict__ count) {
    if (index && (int)(blockIdx.x * CH) >= *count) return;
    __shared__ MogiSrc s_src[CH][NSRC];
    __shared__ int s_chain[CH];
    __shared__ float s_off[CH][kMaxOffsets];
    __shared__ int s_act[CH];
    __shared__ double s_part[CH][8];
    const int c0 = blockIdx.x * CH;
    const double PI = 3.14159265358979323846;
    const int nslots = index ? min(n, *count) : n;
    for (int c = threadIdx.x; c < CH; c += blockDim.x) {
        const int slot = c0 + c;
        s_chain[c] = (slot < nslots) ? (index ? index[slot] : slot) : n;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < CH * NSRC; k += blockDim.x) {
        const int c = k / NSRC, src = k % NSRC, i = s_chain[c];
        MogiSrc S{};
        if (i < n) {
            const double* th = theta + (size_t)i * L.nparams + src * L.source_stride;
            split_hilo(th[L.x_idx], S.pos.x, S.pos.y);
            split_hilo(th[L.x_idx + 1], S.pos.z, S.pos.w);
            const double dv = L.log_strength ? pow(10.0, th[L.strength_idx]) : th[L.strength_idx];
            S.prm = make_float4((float)th[L.depth_idx], (float)((L.nu - 1.0) * dv / PI), 0.f, 0.f);
        }
        s_src[c][src] = S;
    }
    for (int k = threadIdx.x; k < CH * kMaxOffsets; k += blockDim.x) {
        const int c = k / kMaxOffsets, o = k % kMaxOffsets, i = s_chain[c];
        s_off[c][o] = (i < n && o < noffsets)
                          ? (float)theta[(size_t)i * L.nparams + L.offset_idx + o] : 0.f;
    }
    for (int c = threadIdx.x; c < CH; c += blockDim.x) {
        const int i = s_chain[c];
        s_act[c] = (i < n) && !(mask_in && mask_in[i]);
    }
    __syncthreads();
    ff acc[CH];
#pragma unroll
    for (int c = 0; c < CH; ++c) acc[c] = ff{0.f, 0.f};
    for (int j = threadIdx.x; j < m_padded; j += blockDim.x) {
        const float4 A = __ldg(xy + j);
        const float4 B = __ldg(losd + j);
        const float w = __ldg(wt + j);
        const int o = oid ? (__ldg(oid + j) & (kMaxOffsets - 1)) : 0;
#pragma unroll
        for (int c = 0; c < CH; ++c) {
            float u = 0.f;
#pragma unroll
            for (int sidx = 0; sidx < NSRC; ++sidx) {
                const MogiSrc S = s_src[c][sidx];
                // source minus observation point (libmogi/Source.cc:86-88)
                const float dx = (S.pos.x - A.x) + (S.pos.y - A.y);
                const float dy = (S.pos.z - A.z) + (S.pos.w - A.w);
                const float d = S.prm.x;
                const float R2 = fmaf(dx, dx, fmaf(dy, dy, d * d));
                const float iR = rsqrtf(R2);
                const float iR3 = iR * iR * iR;
                const float proj = fmaf(dx, B.x, fmaf(dy, B.y, -d * B.z));
                u = fmaf(S.prm.y * proj, iR3, u);
            }
            float r = u - B.w;
            if (oid) r -= s_off[c][o];
            if (w != 0.f) ff_add_wsq(acc[c], r, w);
            if (resid && s_chain[c] < n) resid[(size_t)s_chain[c] * m_padded + j] = (j < m) ? r : 0.f;
        }
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < CH; ++c) {
        const double v = warp_sum(ff_to_double(acc[c]));
        if (lane == 0) s_part[c][warp] = v;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < CH; c += blockDim.x) {
        if (!s_act[c]) continue;
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += s_part[c][k];
        llk[s_chain[c]] = norm - 0.5 * s;
    }
}

}  // namespace ag

// ---------------------------------------------------------------------------
// C ABI
using namespace ag;

// CDM launch variants: warps (= chains) per CTA and resident CTAs per SM the
// register allocation targets; chosen per problem by the autotuner
struct CdmVariant { int warps; };
static constexpr CdmVariant kCdmVariants[] = {{8}, {4}, {4}, {2}, {4}, {4}, {2}, {4}, {4}, {4}, {4}};
static constexpr int kCdmVariantCount = 11;
static constexpr int kMogiChains = 16;

extern "C" int32_t ag_forward_variants(int model) { return model == AG_MODEL_CDM ? kCdmVariantCount : 1; }

// CDM workspace: compacted chain constants, the chain of each slot, the slot count
static size_t al256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" size_t ag_forward_workspace_bytes(int model, int32_t n) {
    if (model == AG_MODEL_CDM && n > 0)
        return al256((size_t)n * sizeof(ChainC)) + al256((size_t)n * sizeof(int32_t)) + 256;
    return 0;
}

static int check_stations(const ag_station_set* st) {
    AG_REQUIRE(st != nullptr, "stations is NULL");
    AG_REQUIRE(st->xy && st->losd && st->weight, "station arrays must not be NULL");
    AG_REQUIRE(st->m > 0 && st->m_padded >= st->m && st->m_padded % AG_STATION_TILE == 0,
               "m=%d m_padded=%d: m_padded must be a multiple of %d and >= m", st->m,
               st->m_padded, AG_STATION_TILE);
    AG_REQUIRE(aligned(st->xy, 16) && aligned(st->losd, 16) && aligned(st->weight, 16) &&
                   (st->oid == nullptr || aligned(st->oid, 16)),
               "station arrays must be 16-byte aligned");
    return AG_OK;
}

static int forward_llk(int model, const ag_layout* layout, const double* theta, int32_t n,
                       const ag_station_set* st, double norm, const uint32_t* mask_in,
                       const int32_t* index, const int32_t* count, double* llk,
                       uint32_t* chain_status, float* residuals, void* workspace,
                       size_t workspace_bytes, void* stream) {
    AG_REQUIRE(layout != nullptr && theta != nullptr && llk != nullptr, "null argument");
    AG_REQUIRE(n > 0, "n must be positive (got %d)", n);
    int rc = check_stations(st);
    if (rc) return rc;
    const ag_layout L = *layout;
    AG_REQUIRE(L.nparams > 0 && L.x_idx >= 0 && L.x_idx + 1 < L.nparams && L.depth_idx >= 0 &&
                   L.depth_idx < L.nparams && L.strength_idx >= 0 && L.strength_idx < L.nparams,
               "invalid parameter layout");
    int noffsets = 0;
    if (st->oid) {
        AG_REQUIRE(L.offset_idx >= 0, "stations carry dataset ids but the layout has no offsets");
        noffsets = L.nparams - L.offset_idx;
        AG_REQUIRE(noffsets > 0 && noffsets <= kMaxOffsets,
                   "between 1 and %d offset parameters are supported", kMaxOffsets);
    }
    cudaStream_t s = as_stream(stream);
    const float4* xy = reinterpret_cast<const float4*>(st->xy);
    const float4* ld = reinterpret_cast<const float4*>(st->losd);
    if (model == AG_MODEL_CDM) {
        AG_REQUIRE(L.axes_idx >= 0 && L.axes_idx + 2 < L.nparams && L.omega_idx >= 0 &&
                       L.omega_idx + 2 < L.nparams,
                   "invalid CDM layout");
        const size_t need = ag_forward_workspace_bytes(model, n);
        AG_REQUIRE(workspace != nullptr && workspace_bytes >= need && aligned(workspace, 256),
                   "CDM needs %zu bytes of 256-byte aligned workspace", need);
        ChainC* chains = reinterpret_cast<ChainC*>(workspace);
        int32_t* slot_chain = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) +
                                                         al256((size_t)n * sizeof(ChainC)));
        int32_t* nslots = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(slot_chain) +
                                                     al256((size_t)n * sizeof(int32_t)));
        rc = cuda_status(cudaMemsetAsync(nslots, 0, sizeof(int32_t), s), "cudaMemsetAsync(slot count)");
        if (rc) return rc;
        cdm_setup_kernel<<<(n + 127) / 128, 128, 0, s>>>(L, theta, n, mask_in, chains, chain_status, noffsets,
                                                         index, count, slot_chain, nslots);
        rc = launch_status("cdm_setup_kernel");
        if (rc) return rc;
        const int v = L.variant;
        AG_REQUIRE(v >= 0 && v < kCdmVariantCount, "CDM variant %d out of range [0, %d)", v, kCdmVariantCount);
        const int warps = kCdmVariants[v].warps;
        const int grid = (n + warps - 1) / warps;
#define AG_CDM_LAUNCH(W, B, SPL)                                                                    \
    cdm_llk_kernel<W, B, SPL><<<grid, W * 32, 0, s>>>(chains, slot_chain, nslots, n, xy, ld, st->weight, \
                                                      st->oid, st->m, st->m_padded, norm, llk, residuals, nullptr)
        switch (v) {
            case 0: AG_CDM_LAUNCH(8, 2, 1); break;
            case 1: AG_CDM_LAUNCH(4, 4, 1); break;
            case 2: AG_CDM_LAUNCH(4, 5, 1); break;
            case 3: AG_CDM_LAUNCH(2, 8, 1); break;
            case 4: AG_CDM_LAUNCH(4, 3, 2); break;
            case 5: AG_CDM_LAUNCH(4, 4, 2); break;
            case 6: AG_CDM_LAUNCH(2, 6, 2); break;
            case 7: AG_CDM_LAUNCH(4, 2, 4); break;
            case 8: AG_CDM_LAUNCH(4, 3, 4); break;
            case 9: AG_CDM_LAUNCH(4, 4, 4); break;
            default: AG_CDM_LAUNCH(4, 5, 4); break;
        }
#undef AG_CDM_LAUNCH
        return launch_status("cdm_llk_kernel");
    }
    if (model == AG_MODEL_MOGI) {
        AG_REQUIRE(L.nsources == 1 || L.nsources == 2, "1 or 2 Mogi sources are supported");
        const int grid = (n + kMogiChains - 1) / kMogiChains;
        if (L.nsources == 1)
            mogi_llk_kernel<kMogiChains, 1><<<grid, 256, 0, s>>>(
                L, theta, n, mask_in, xy, ld, st->weight, st->oid, noffsets, st->m, st->m_padded, norm, llk,
                residuals, index, count);
        else
            mogi_llk_kernel<kMogiChains, 2><<<grid, 256, 0, s>>>(
                L, theta, n, mask_in, xy, ld, st->weight, st->oid, noffsets, st->m, st->m_padded, norm, llk,
                residuals, index, count);
        return launch_status("mogi_llk_kernel");
    }
    return set_error(AG_ERR_ARG, "unknown model %d", model);
}

extern "C" int ag_forward_llk(int model, const ag_layout* layout, const double* theta, int32_t n,
                              const ag_station_set* st, double norm, const uint32_t* mask_in,
                              double* llk, uint32_t* chain_status, float* residuals,
                              void* workspace, size_t workspace_bytes, void* stream) {
    return forward_llk(model, layout, theta, n, st, norm, mask_in, nullptr, nullptr, llk, chain_status,
                       residuals, workspace, workspace_bytes, stream);
}

extern "C" int ag_forward_llk_subset(int model, const ag_layout* layout, const double* theta,
                                     int32_t n, const ag_station_set* st, double norm,
                                     const int32_t* index, const int32_t* count, double* llk,
                                     uint32_t* chain_status, float* residuals, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    AG_REQUIRE(index != nullptr && count != nullptr, "index and count must not be NULL");
    return forward_llk(model, layout, theta, n, st, norm, nullptr, index, count, llk, chain_status,
                       residuals, workspace, workspace_bytes, stream);
}

extern "C" int ag_cdm_check(const ag_layout* layout, const double* theta, int32_t n,
                            uint32_t* chain_status, void* stream) {
    AG_REQUIRE(layout && theta && chain_status && n > 0, "invalid arguments");
    cdm_check_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(*layout, theta, n, chain_status);
    return launch_status("cdm_check_kernel");
}
