// Shared device utilities for the CATMIP kernels (sm_103a).
//
// * Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
//   "Parallel random numbers: as easy as 1, 2, 3", SC 2011), so that every
//   random draw is a pure function of (seed, chain, stream, step, epoch) and
//   the CPU oracle can reproduce it bit for bit.
// * float-float ("double-single") accumulation built from the error-free
//   transformations TwoSum (Knuth) and TwoProd via FMA, used for the per-chain
//   misfit sums so that the FP64 log-likelihood is exact to ~1e-14 of the FP32
//   residuals it sums.
// * bounded mbarrier waits: every wait gives up after a fixed number of
//   polls and raises an error flag instead of spinning forever.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef AG_DEVICE_INLINE
#define AG_DEVICE_INLINE __device__ __forceinline__
#endif

namespace ag {

// ---------------------------------------------------------------------------
// error flags written by kernels into a caller-provided device word
enum : uint32_t {
    DEV_ERR_TIMEOUT = 1u,      // a bounded wait gave up
    DEV_ERR_NOT_SPD = 2u,      // Cholesky met a non-positive pivot
    DEV_ERR_NONFINITE = 4u,    // a non-finite value where none may appear
};

// per-chain status bits (mirror the public header)
enum : uint32_t {
    CHAIN_OUT_OF_SUPPORT = 1u,
    CHAIN_ABOVE_SURFACE = 2u,
    CHAIN_NONFINITE = 4u,
};

AG_DEVICE_INLINE void raise_flag(uint32_t* flag, uint32_t bits) {
    if (flag) atomicOr(flag, bits);
}

// ---------------------------------------------------------------------------
// Philox4x32-10
struct u32x4 { uint32_t x, y, z, w; };

AG_DEVICE_INLINE void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    lo = a * b;
    hi = __umulhi(a, b);
}

AG_DEVICE_INLINE u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
    // round multipliers and Weyl key increments from the Philox paper
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo(M0, c.x, hi0, lo0);
        mulhilo(M1, c.z, hi1, lo1);
        u32x4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// random streams: the third counter word carries the stream tag in its top byte
enum : uint32_t {
    STREAM_PRIOR = 0u,
    STREAM_PROPOSAL = 1u,
    STREAM_ACCEPT = 2u,
    STREAM_RESAMPLE = 3u,
};

AG_DEVICE_INLINE u32x4 draw(uint64_t seed, uint32_t unit, uint32_t sub, uint32_t stream,
                            uint32_t step, uint32_t epoch) {
    u32x4 c{unit, sub, (stream << 24) | (step & 0x00FFFFFFu), epoch};
    return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// 53-bit integer from two words: (a >> 5) * 2^26 + (b >> 6)
AG_DEVICE_INLINE uint64_t bits53(uint32_t a, uint32_t b) {
    return ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
}
// uniform on [0, 1)
AG_DEVICE_INLINE double u01_closed_open(uint32_t a, uint32_t b) {
    return (double)bits53(a, b) * 0x1.0p-53;
}
// uniform on (0, 1]
AG_DEVICE_INLINE double u01_open_closed(uint32_t a, uint32_t b) {
    return (double)(bits53(a, b) + 1ull) * 0x1.0p-53;
}

// Box-Muller pair from one Philox block
AG_DEVICE_INLINE void normal_pair(u32x4 r, double& z0, double& z1) {
    double u1 = u01_open_closed(r.x, r.y);
    double u2 = u01_closed_open(r.z, r.w);
    double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    z0 = rad * c;
    z1 = rad * s;
}

// ---------------------------------------------------------------------------
// float-float accumulation
struct ff { float hi, lo; };

AG_DEVICE_INLINE void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// acc += x (x given as an unevaluated sum xh + xl)
AG_DEVICE_INLINE void ff_add(ff& acc, float xh, float xl) {
    float s, e;
    two_sum(acc.hi, xh, s, e);
    e += acc.lo + xl;
    float h = s + e;
    acc.lo = e - (h - s);
    acc.hi = h;
}

// acc += w * r * r, exact products via FMA
AG_DEVICE_INLINE void ff_add_wsq(ff& acc, float r, float w) {
    float p = r * r;
    float pe = fmaf(r, r, -p);            // r*r = p + pe exactly
    float q = p * w;
    float qe = fmaf(p, w, -q) + pe * w;   // (p + pe) * w ~= q + qe
    ff_add(acc, q, qe);
}

AG_DEVICE_INLINE double ff_to_double(const ff& a) { return (double)a.hi + (double)a.lo; }

// warp sum of doubles (fixed butterfly order: deterministic)
AG_DEVICE_INLINE double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// bounded mbarrier helpers (shared::cta)
AG_DEVICE_INLINE uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

AG_DEVICE_INLINE void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

AG_DEVICE_INLINE void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

AG_DEVICE_INLINE void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

AG_DEVICE_INLINE bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(smem_addr(bar)), "r"(phase) : "memory");
    return ok != 0;
}

// Wait for the given phase parity; gives up after `limit` polls (each poll
// itself blocks for a hardware-defined slice) and reports false.
AG_DEVICE_INLINE bool mbar_wait_bounded(uint64_t* bar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// order this thread's earlier shared-memory accesses (generic proxy) before the
// asynchronous copies it issues next
AG_DEVICE_INLINE void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 1-D bulk copy global -> shared (16-byte aligned, size multiple of 16),
// completion signalled on `bar` through the transaction count.
AG_DEVICE_INLINE void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

}  // namespace ag
