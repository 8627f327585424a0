// Linear Gaussian model on the 5th-generation tensor cores (tcgen05).
//
// The reference's linear model (models/linear/linear/Linear.py:152-185) forms
// r = G θ - d with a dgemm and whitens each chain's residual.  Here the data
// covariance is folded once into A = L⁻¹ G and b = L⁻¹ d (Cd = L Lᵀ), so that
// rᵀ Cd⁻¹ r = |A θ - b|², and each chain's misfit is
//     ρ = A (θ - θ₀) + ρ₀,   ρ₀ = A θ₀ - b  (FP64, the residual-correction pass),
// with θ₀ a centre of the population (the mean of up to 256 evenly spaced
// chains): the tensor-core product only carries the centred part.  A and
// δ = θ - θ₀ are split into BF16 pairs (x ≈ hi + lo) and
// the product A δ is one GEMM over the concatenated K axis
//     [δ_hi | δ_lo | δ_hi] · [A_hi | A_hi | A_lo]ᵀ
// (three BF16 products, FP32 accumulation; the dropped lo·lo term is
// ~2^-18 relative).  The GEMM is a persistent tcgen05 kernel: TMA loads
// 128B-swizzled K-major tiles into a 4-stage shared-memory ring guarded by
// mbarriers, one thread issues tcgen05.mma (M = 128 chains, N = 256
// observations, K = 16) into one of two TMEM accumulators, and four epilogue
// warps read the other accumulator with tcgen05.ld and reduce Σ (acc + ρ₀)²
// per chain straight from registers while the next tile's MMAs run.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"
#include "tcgen05.cuh"

namespace ag {

// Persistent CTAs, one per SM, each taking tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...
// of 128 chains x 256 observations; partial[tile_n * n + chain] = Σ_obs (acc + ρ₀)².
// Warp roles: warp 0 lane 0 drives TMA through the TC_STAGES shared-memory ring, warp 1
// lane 0 issues tcgen05.mma into one of two TMEM accumulators (2 x 256 columns), warps
// 2-5 read the other accumulator with tcgen05.ld and reduce the previous tile, so the
// epilogue and the next tile's MMAs overlap.  Tiles are visited in groups of
// TC_GROUP_M chain tiles so that CTAs running at the same time share both operands' k
// slices in L2.  Every wait is bounded; a timeout stops all roles, drains the copies
// and MMAs in flight and frees TMEM.
constexpr int TC_THREADS = 192;
constexpr int TC_GROUP_M = 8;
constexpr uint32_t TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 /*align*/ + 256 /*bars*/;

AG_DEVICE_INLINE void tile_coords(int t, int mtiles, int ntiles, int& mt, int& nt) {
    const int span = TC_GROUP_M * ntiles;
    const int g = t / span, r = t % span;
    const int gm = (mtiles - g * TC_GROUP_M) < TC_GROUP_M ? (mtiles - g * TC_GROUP_M) : TC_GROUP_M;
    mt = g * TC_GROUP_M + r % gm;
    nt = r / gm;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
linear_misfit_tc_kernel(const __grid_constant__ CUtensorMap map_a,   // chains  x K' (BF16)
                        const __grid_constant__ CUtensorMap map_b,   // obs     x K' (BF16)
                        int n, int m_obs, int kblocks, int mtiles, int ntiles,
                        const float* __restrict__ rho0, double* __restrict__ partial,
                        uint32_t* __restrict__ flags) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + TC_STAGES * TC_STAGE_BYTES);
    uint64_t* full = bars;                       // [TC_STAGES]  TMA -> MMA
    uint64_t* empty = bars + TC_STAGES;          // [TC_STAGES]  MMA -> TMA
    uint64_t* tfull = bars + 2 * TC_STAGES;      // [2]          MMA -> epilogue
    uint64_t* tempty = bars + 2 * TC_STAGES + 2; // [2]          epilogue -> MMA
    uint64_t* drain = bars + 2 * TC_STAGES + 4;  // [1]          all MMAs done (teardown)
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = mtiles * ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 4);
        }
        mbar_init(drain, 1);
        fence_mbar_init();
        s_abort = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_addr(&s_tmem)), "r"(2 * TC_BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    auto aborted = [&]() { return *(volatile int*)&s_abort != 0; };

    int issued = 0;                              // TMA stages issued (producer thread)
    if (warp == 0 && lane == 0) {
        // TMA producer: the stage ring runs on across tiles
        for (int t = blockIdx.x; t < total && !aborted(); t += gridDim.x) {
            int mt, nt;
            tile_coords(t, mtiles, ntiles, mt, nt);
            for (int kb = 0; kb < kblocks; ++kb, ++issued) {
                const int s = issued % TC_STAGES;
                if (issued >= TC_STAGES &&
                    !mbar_wait_bounded(&empty[s], (uint32_t)((issued / TC_STAGES) - 1) & 1u, TC_WAIT)) {
                    atomicExch(&s_abort, 1);
                    break;
                }
                if (aborted()) break;
                const uint32_t sa = base + s * TC_STAGE_BYTES;
                mbar_arrive_expect_tx(&full[s], TC_STAGE_BYTES);
                tma_load_2d(sa, &map_a, kb * TC_BK, mt * TC_BM, smem_addr(&full[s]));
                tma_load_2d(sa + TC_A_BYTES, &map_b, kb * TC_BK, nt * TC_BN, smem_addr(&full[s]));
            }
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: tile j of this CTA accumulates into TMEM columns (j & 1) * 256
        const uint32_t idesc = idesc_bf16(TC_BM, TC_BN);
        int it = 0, local = 0;
        for (int t = blockIdx.x; t < total && !aborted(); t += gridDim.x, ++local) {
            const int b = local & 1;
            if (local >= 2 && !mbar_wait_bounded(&tempty[b], (uint32_t)((local >> 1) - 1) & 1u, TC_WAIT)) {
                atomicExch(&s_abort, 1);
                break;
            }
            tc_fence_after();
            const uint32_t acc_addr = tmem + (uint32_t)(b * TC_BN);
            bool ok = true;
            for (int kb = 0; kb < kblocks; ++kb, ++it) {
                const int s = it % TC_STAGES;
                if (!mbar_wait_bounded(&full[s], (uint32_t)(it / TC_STAGES) & 1u, TC_WAIT)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = base + s * TC_STAGE_BYTES;
                const uint64_t adesc = sw128_desc(sa), bdesc = sw128_desc(sa + TC_A_BYTES);
#pragma unroll
                for (int k = 0; k < TC_BK / 16; ++k)   // K = 16 per instruction: +32 bytes
                    mma_bf16(acc_addr, adesc + 2 * k, bdesc + 2 * k, idesc, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(smem_addr(&empty[s]));
            }
            if (!ok) {
                atomicExch(&s_abort, 1);
                break;
            }
            mma_commit(smem_addr(&tfull[b]));    // fires when this tile's MMAs have completed
        }
        mma_commit(smem_addr(drain));            // fires when every issued MMA has completed
    } else if (warp >= 2) {
        // epilogue: thread = chain row (TMEM lane quarter of this warp), sums over observations
        const int quarter = warp & 3;
        const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
        int local = 0;
        for (int t = blockIdx.x; t < total; t += gridDim.x, ++local) {
            const int b = local & 1;
            const bool ok = __all_sync(0xffffffffu,
                                       mbar_wait_bounded(&tfull[b], (uint32_t)(local >> 1) & 1u, TC_WAIT));
            if (!ok || aborted()) {
                if (lane == 0) atomicExch(&s_abort, 1);
                break;
            }
            tc_fence_after();
            int mt, nt;
            tile_coords(t, mtiles, ntiles, mt, nt);
            const int n0 = nt * TC_BN;
            const int chain = mt * TC_BM + quarter * 32 + lane;
            double acc = 0.0;
#pragma unroll 1
            for (int c0 = 0; c0 < TC_BN; c0 += 64) {
                // two 32-column loads in flight per wait; lane l holds ρ₀ of observation
                // n0 + c0 + l (and + 32), broadcast by shuffles
                uint32_t r0[32], r1[32];
                tmem_ld32_nowait(tmem + lane_base + (uint32_t)(b * TC_BN + c0), r0);
                tmem_ld32_nowait(tmem + lane_base + (uint32_t)(b * TC_BN + c0 + 32), r1);
                const int obs_l = n0 + c0 + lane;
                const float rho_a = (obs_l < m_obs) ? __ldg(rho0 + obs_l) : 0.f;
                const float rho_b = (obs_l + 32 < m_obs) ? __ldg(rho0 + obs_l + 32) : 0.f;
                tmem_wait_ld();
                float sq = 0.f;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float r = __uint_as_float(r0[i]) + __shfl_sync(0xffffffffu, rho_a, i);
                    sq = (n0 + c0 + i < m_obs) ? fmaf(r, r, sq) : sq;
                }
                acc += (double)sq;
                sq = 0.f;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float r = __uint_as_float(r1[i]) + __shfl_sync(0xffffffffu, rho_b, i);
                    sq = (n0 + c0 + 32 + i < m_obs) ? fmaf(r, r, sq) : sq;
                }
                acc += (double)sq;
            }
            if (chain < n) partial[(size_t)nt * n + chain] = acc;
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && aborted()) raise_flag(flags, DEV_ERR_TIMEOUT);
    if (warp == 0 && lane == 0 && aborted()) {
        // copies still in flight land before the CTA's shared memory goes away
        for (int k = (issued > TC_STAGES ? issued - TC_STAGES : 0); k < issued; ++k)
            mbar_wait_bounded(&full[k % TC_STAGES], (uint32_t)(k / TC_STAGES) & 1u, TC_WAIT);
    }
    if (warp == 1) {
        // every MMA this CTA issued has completed before TMEM is released
        mbar_wait_bounded(drain, 0, TC_WAIT);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BN) : "memory");
    }
}

// ρ₀ = W r̄ in FP64 (one warp per whitened observation)
__global__ void whiten_rho0_kernel(const double* __restrict__ W, const double* __restrict__ mean, int m,
                                   float* __restrict__ rho0) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= m) return;
    double s = 0.0;
    for (int j = lane; j < m; j += 32) s = fma(W[(size_t)row * m + j], mean[j], s);
    s = warp_sum(s);
    if (lane == 0) rho0[row] = (float)s;
}

// θ₀ = column means of θ (one thread per parameter, fixed order)
// Centring point θ₀ (or r̄): the mean of up to kCentreRows rows taken at an even stride.
// Any centre gives the same result, because ρ₀ = A θ₀ - b carries it exactly in FP64;
// the centre only has to lie inside the population so that the BF16 split of θ - θ₀ keeps
// its relative precision.  One thread per column, rows in a fixed order.
constexpr int kCentreRows = 256;
static inline int cdiv(long a, long b) { return (int)((a + b - 1) / b); }

template <class T>
__global__ void __launch_bounds__(256) centre_kernel(const T* __restrict__ x, int ld, int col0, int n, int cols,
                                                     double* __restrict__ centre) {
    // 32 columns per CTA (lanes), the sampled rows split over the 8 warps, then the warp
    // partial sums added in warp order
    __shared__ double part[8][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    const int rows = n < kCentreRows ? n : kCentreRows;
    const long stride = n / rows;                      // >= 1
    double s = 0.0;
    if (j < cols) {
#pragma unroll 4
        for (int k = warp; k < rows; k += 8) s += (double)__ldg(x + (size_t)(k * stride) * ld + col0 + j);
    }
    part[warp][lane] = s;
    __syncthreads();
    if (warp == 0 && j < cols) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += part[w][lane];
        centre[j] = t / rows;
    }
}

// ρ₀ = A θ₀ - b in FP64 (one warp per observation)
__global__ void rho0_kernel(const double* __restrict__ A, const double* __restrict__ b,
                            const double* __restrict__ theta0, int m, int p, float* __restrict__ rho0) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (row >= m) return;
    double s = 0.0;
    for (int j = lane; j < p; j += 32) s = fma(A[(size_t)row * p + j], theta0[j], s);
    s = warp_sum(s);
    if (lane == 0) rho0[row] = (float)(s - b[row]);
}

// δ = x - centre split as [hi | lo | hi] (BF16, row length 3 kp, kp = columns padded to
// 64): one thread per 8 consecutive columns of a row, three 16-byte stores.  Rows of x have
// stride ld and start at column col0 (θ: ld = p, col0 = 0; a residual block: the residual
// rows and the block's first column).
template <class T>
__global__ void split_centred_kernel(const T* __restrict__ x, int ld, int col0, const double* __restrict__ centre,
                                     int n, int cols, int kp, __nv_bfloat16* __restrict__ out) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int groups = kp >> 3;
    if (e >= (long)n * groups) return;
    const int i = (int)(e / groups), j0 = (int)(e % groups) * 8;
    __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const int j = j0 + q;
        const float d = (j < cols) ? (float)((double)x[(size_t)i * ld + col0 + j] - centre[j]) : 0.f;
        hi[q] = __float2bfloat16_rn(d);
        lo[q] = __float2bfloat16_rn(d - __bfloat162float(hi[q]));
    }
    __nv_bfloat16* row = out + (size_t)i * 3 * kp;
    const uint4 h = *reinterpret_cast<const uint4*>(hi), l = *reinterpret_cast<const uint4*>(lo);
    *reinterpret_cast<uint4*>(row + j0) = h;
    *reinterpret_cast<uint4*>(row + kp + j0) = l;
    *reinterpret_cast<uint4*>(row + 2 * kp + j0) = h;
}

// A split as [hi | hi | lo]
__global__ void split_a_kernel(const double* __restrict__ A, int m, int p, int kp,
                               __nv_bfloat16* __restrict__ out) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)m * kp) return;
    const int i = (int)(e / kp), j = (int)(e % kp);
    const float a = (j < p) ? (float)A[(size_t)i * p + j] : 0.f;
    const __nv_bfloat16 hi = __float2bfloat16_rn(a);
    const __nv_bfloat16 lo = __float2bfloat16_rn(a - __bfloat162float(hi));
    __nv_bfloat16* row = out + (size_t)i * 3 * kp;
    row[j] = hi;
    row[kp + j] = hi;
    row[2 * kp + j] = lo;
}

__global__ void linear_reduce_kernel(int n, int tiles, const double* __restrict__ partial, double norm,
                                     double* __restrict__ llk, int accumulate) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int t = 0; t < tiles; ++t) s += partial[(size_t)t * n + i];
    llk[i] = (accumulate ? llk[i] : norm) - 0.5 * s;
}




// Exact FP64 reference path: ρ = A θ - b per chain (one warp per chain, observations strided)
__global__ void linear_fp64_kernel(const double* __restrict__ A, const double* __restrict__ b,
                                   const double* __restrict__ theta, int n, int m, int p, double norm,
                                   double* __restrict__ llk) {
    const int chain = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (chain >= n) return;
    const double* th = theta + (size_t)chain * p;
    double acc = 0.0;
    for (int r = lane; r < m; r += 32) {
        double s = -b[r];
        for (int j = 0; j < p; ++j) s = fma(A[(size_t)r * p + j], th[j], s);
        acc = fma(s, s, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) llk[chain] = norm - 0.5 * acc;
}


}  // namespace ag

using namespace ag;

static inline size_t al256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" int32_t ag_linear_kpad(int32_t p) { return p > 0 ? cdiv(p, TC_BK) * TC_BK : 0; }

extern "C" int ag_linear_prepare(const double* A, int32_t m, int32_t p, uint16_t* a_split, void* stream) {
    AG_REQUIRE(A && a_split && m > 0 && p > 0, "invalid arguments");
    const int kp = ag_linear_kpad(p);
    split_a_kernel<<<cdiv((long)m * kp, 256), 256, 0, as_stream(stream)>>>(A, m, p, kp,
                                                                         reinterpret_cast<__nv_bfloat16*>(a_split));
    return launch_status("split_a_kernel");
}

extern "C" size_t ag_linear_workspace_bytes(int32_t m, int32_t p, int32_t n) {
    if (m <= 0 || p <= 0 || n <= 0) return 0;
    const size_t kp = ag_linear_kpad(p);
    return al256(p * sizeof(double)) + al256((size_t)m * sizeof(float)) +
           al256((size_t)n * 3 * kp * 2) + al256((size_t)cdiv(m, TC_BN) * n * sizeof(double));
}

extern "C" int ag_linear_llk(const ag_linear_model* lm, const double* theta, int32_t n, double norm,
                             double* llk, void* workspace, size_t workspace_bytes, uint32_t* flags,
                             void* stream) {
    AG_REQUIRE(lm && lm->a64 && lm->b64 && lm->a_split && theta && llk && n > 0, "invalid arguments");
    const int m = lm->m_obs, p = lm->p;
    AG_REQUIRE(m > 0 && p > 0, "invalid linear model sizes");
    const size_t need = ag_linear_workspace_bytes(m, p, n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "ag_linear_llk needs %zu bytes of 256-byte aligned workspace", need);
    AG_REQUIRE(aligned(lm->a_split, 16), "a_split must be 16-byte aligned");
    cudaStream_t s = as_stream(stream);
    const int kp = ag_linear_kpad(p);
    char* ws = static_cast<char*>(workspace);
    double* theta0 = reinterpret_cast<double*>(ws); ws += al256(p * sizeof(double));
    float* rho0 = reinterpret_cast<float*>(ws); ws += al256((size_t)m * sizeof(float));
    __nv_bfloat16* tsplit = reinterpret_cast<__nv_bfloat16*>(ws); ws += al256((size_t)n * 3 * kp * 2);
    double* partial = reinterpret_cast<double*>(ws);
    const int tiles = cdiv(m, TC_BN);
    centre_kernel<double><<<cdiv(p, 32), 256, 0, s>>>(theta, p, 0, n, p, theta0);
    rho0_kernel<<<cdiv((long)m * 32, 256), 256, 0, s>>>(lm->a64, lm->b64, theta0, m, p, rho0);
    split_centred_kernel<double><<<cdiv((long)n * (kp / 8), 256), 256, 0, s>>>(theta, p, 0, theta0, n, p, kp,
                                                                                tsplit);
    int rc = launch_status("linear prologue kernels");
    if (rc) return rc;
    CUtensorMap ma, mb;
    rc = make_map(&ma, tsplit, n, 3 * kp, TC_BM);
    if (rc) return rc;
    rc = make_map(&mb, lm->a_split, m, 3 * kp, TC_BN);
    if (rc) return rc;
    // per call: the attribute belongs to the current device's context
    rc = cuda_status(cudaFuncSetAttribute(linear_misfit_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TC_SMEM),
                     "cudaFuncSetAttribute(linear_misfit_tc_kernel)");
    if (rc) return rc;
    const int mtiles = cdiv(n, TC_BM), total = mtiles * tiles;
    int sms = 0;
    rc = sm_count(&sms);
    if (rc) return rc;
    linear_misfit_tc_kernel<<<total < sms ? total : sms, TC_THREADS, TC_SMEM, s>>>(
        ma, mb, n, m, 3 * kp / TC_BK, mtiles, tiles, rho0, partial, flags);
    rc = launch_status("linear_misfit_tc_kernel");
    if (rc) return rc;
    linear_reduce_kernel<<<cdiv(n, 256), 256, 0, s>>>(n, tiles, partial, norm, llk, 0);
    return launch_status("linear_reduce_kernel");
}

extern "C" size_t ag_whiten_workspace_bytes(int32_t m, int32_t n) {
    if (m <= 0 || n <= 0) return 0;
    const size_t kp = ag_linear_kpad(m);
    return al256(m * sizeof(double)) + al256(sizeof(double)) + al256((size_t)m * sizeof(float)) +
           al256((size_t)n * 3 * kp * 2) + al256((size_t)cdiv(m, TC_BN) * n * sizeof(double));
}

extern "C" int ag_whiten_llk(const ag_whiten_block* blk, const float* resid, int32_t ldr, int32_t n,
                             double* llk, void* workspace, size_t workspace_bytes, uint32_t* flags,
                             void* stream) {
    AG_REQUIRE(blk && blk->w64 && blk->w_split && resid && llk && n > 0, "invalid arguments");
    const int m = blk->m, col0 = blk->col0;
    AG_REQUIRE(m > 0 && col0 >= 0 && col0 + m <= ldr, "block columns [%d, %d) outside rows of %d", col0, col0 + m,
               ldr);
    const size_t need = ag_whiten_workspace_bytes(m, n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "ag_whiten_llk needs %zu bytes of 256-byte aligned workspace", need);
    AG_REQUIRE(aligned(blk->w_split, 16), "w_split must be 16-byte aligned");
    cudaStream_t s = as_stream(stream);
    const int kp = ag_linear_kpad(m);
    char* ws = static_cast<char*>(workspace);
    double* mean = reinterpret_cast<double*>(ws); ws += al256(m * sizeof(double));
    ws += al256(sizeof(double));
    float* rho0 = reinterpret_cast<float*>(ws); ws += al256((size_t)m * sizeof(float));
    __nv_bfloat16* rsplit = reinterpret_cast<__nv_bfloat16*>(ws); ws += al256((size_t)n * 3 * kp * 2);
    double* partial = reinterpret_cast<double*>(ws);
    const int tiles = cdiv(m, TC_BN);
    centre_kernel<float><<<cdiv(m, 32), 256, 0, s>>>(resid, ldr, col0, n, m, mean);
    int rc = launch_status("whitening prologue");
    if (rc) return rc;
    split_centred_kernel<float><<<cdiv((long)n * (kp / 8), 256), 256, 0, s>>>(resid, ldr, col0, mean, n, m, kp,
                                                                              rsplit);
    rc = launch_status("split_centred_kernel");
    if (rc) return rc;
    CUtensorMap ma, mb;
    rc = make_map(&ma, rsplit, n, 3 * kp, TC_BM);
    if (rc) return rc;
    rc = make_map(&mb, blk->w_split, m, 3 * kp, TC_BN);
    if (rc) return rc;
    rc = cuda_status(cudaFuncSetAttribute(linear_misfit_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)TC_SMEM),
                     "cudaFuncSetAttribute(linear_misfit_tc_kernel)");
    if (rc) return rc;
    whiten_rho0_kernel<<<cdiv((long)m * 32, 256), 256, 0, s>>>(blk->w64, mean, m, rho0);
    rc = launch_status("whiten_rho0_kernel");
    if (rc) return rc;
    const int mtiles = cdiv(n, TC_BM), total = mtiles * tiles;
    int sms = 0;
    rc = sm_count(&sms);
    if (rc) return rc;
    linear_misfit_tc_kernel<<<total < sms ? total : sms, TC_THREADS, TC_SMEM, s>>>(
        ma, mb, n, m, 3 * kp / TC_BK, mtiles, tiles, rho0, partial, flags);
    rc = launch_status("linear_misfit_tc_kernel (whitening)");
    if (rc) return rc;
    linear_reduce_kernel<<<cdiv(n, 256), 256, 0, s>>>(n, tiles, partial, 0.0, llk, 1);
    return launch_status("linear_reduce_kernel (whitening)");
}

extern "C" int ag_linear_llk_fp64(const ag_linear_model* lm, const double* theta, int32_t n, double norm,
                                  double* llk, void* stream) {
    AG_REQUIRE(lm && lm->a64 && lm->b64 && theta && llk && n > 0, "invalid arguments");
    linear_fp64_kernel<<<cdiv((long)n * 32, 256), 256, 0, as_stream(stream)>>>(lm->a64, lm->b64, theta, n,
                                                                             lm->m_obs, lm->p, norm, llk);
    return launch_status("linear_fp64_kernel");
}
