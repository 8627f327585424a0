// Learned surrogate of the CDM LOS field and the delayed-acceptance steps.
//
// Network: dense layers y = x Wᵀ + b with GELU (x Φ(x)) between them and a
// linear output; weights kept as an FP32 master copy for Adam plus a BF16 copy
// that the forward and backward products read (FP32 accumulation).  Layer
// products are a tiled SIMT GEMM with fused bias / GELU epilogues.
//
// Surrogate log-likelihood: the network predicts K normalised PCA coefficients
// c of the LOS field; with the basis B (M x K), mean field μ and the diagonal
// weights W = Cd⁻¹, Σ_j w_j (ũ_j - d_j)² for ũ = μ + B diag(s) c is
//     q0 - 2 hᵀ c̃ + c̃ᵀ G c̃,  c̃ = s ⊙ c,  h = Bᵀ W (d - μ),  G = Bᵀ W B,
// so each chain costs O(K²) instead of O(M).
//
// Delayed acceptance (Christen & Fox 2005): stage 1 accepts the proposal on
// the surrogate posterior; only stage-1 survivors (compacted into an index
// list) get the exact likelihood; stage 2 accepts with
//     log u2 <= (post' - post) - (post̃' - post̃),
// which leaves the exact posterior invariant.
#include <math.h>
#include <stdint.h>
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include "common.cuh"
#include "internal.h"
#include "tcgen05.cuh"

namespace cg = cooperative_groups;

namespace ag {

constexpr int kMaxLayers = 8;
constexpr int BM = 64, BN = 64, BK = 16;

AG_DEVICE_INLINE float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
AG_DEVICE_INLINE float gelu_grad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) +
           z * 0.39894228040143268f * __expf(-0.5f * z * z);
}

enum Epilogue : int { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2 };

// C(m, n) = Σ_k A(m, k) B(k, n) with A(m,k) = A[m*sam + k*sak], B(k,n) = B[k*sbk + n*sbn]
// (B in BF16 or FP32), then the epilogue: + bias[n], GELU (pre-activation to Z).
//
// 64 x 64 output tile per CTA, 256 threads with 4 x 4 outputs each, k-tiles of 16 staged in
// shared memory; each operand is read along whichever of its two strides is 1 (coalesced
// rows of 16 k or of 64 m / n) and the next k-tile is prefetched into registers while the
// current one is multiplied.  Split K: the gridDim.z CTAs of one tile form a thread-block
// cluster, each multiplies one K range, and the partial tiles are summed through
// distributed shared memory in rank order (deterministic), each CTA reducing and writing
// BM / gridDim.z rows.
template <bool B_BF16>
AG_DEVICE_INLINE float load_b(const void* Bv, long idx) {
    return B_BF16 ? __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(Bv)[idx])
                  : reinterpret_cast<const float*>(Bv)[idx];
}

template <bool B_BF16>
__global__ void __launch_bounds__(256) gemm_kernel(int M, int N, int K, const float* __restrict__ A,
                                                   long sam, long sak, const void* __restrict__ Bv,
                                                   long sbk, long sbn, float* __restrict__ C, long ldc,
                                                   const float* __restrict__ bias, int epi,
                                                   float* __restrict__ Z) {
    __shared__ __align__(16) float As[BK][BM + 4];
    __shared__ __align__(16) float Bs[BK][BN + 4];
    __shared__ __align__(16) float Ps[BM][BN];          // partial tile (split K)
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int split = gridDim.z, part = blockIdx.z;
    const int kchunk = ((K + split - 1) / split + BK - 1) / BK * BK;
    const int kb = min(K, part * kchunk), ke = min(K, kb + kchunk);
    // element e of a 16 x 64 operand tile: (k, m) with k fastest when that stride is 1
    const bool a_k1 = (sak == 1), b_k1 = (sbk == 1);
    float ra[4], rb[4];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + 256 * q;
            int kk = a_k1 ? e % BK : e / BM, mm = a_k1 ? e / BK : e % BM;
            int m = m0 + mm, k = k0 + kk;
            ra[q] = (m < M && k < ke) ? A[(long)m * sam + (long)k * sak] : 0.f;
            kk = b_k1 ? e % BK : e / BN;
            const int nn = b_k1 ? e / BK : e % BN;
            const int n = n0 + nn;
            k = k0 + kk;
            rb[q] = (n < N && k < ke) ? load_b<B_BF16>(Bv, (long)k * sbk + (long)n * sbn) : 0.f;
        }
    };
    auto stash = [&]() {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + 256 * q;
            As[a_k1 ? e % BK : e / BM][a_k1 ? e / BK : e % BM] = ra[q];
            Bs[b_k1 ? e % BK : e / BN][b_k1 ? e / BK : e % BN] = rb[q];
        }
    };
    float acc[4][4] = {};
    if (kb < ke) fetch(kb);
    for (int k0 = kb; k0 < ke; k0 += BK) {
        stash();
        __syncthreads();
        if (k0 + BK < ke) fetch(k0 + BK);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
            const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
    auto store = [&](int m, int n, float v) {
        if (m >= M || n >= N) return;
        if (epi != EPI_NONE) v += bias[n];
        if (epi == EPI_BIAS_GELU) {
            Z[(long)m * ldc + n] = v;
            v = gelu(v);
        }
        C[(long)m * ldc + n] = v;
    };
    if (split == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) store(m0 + ty * 4 + i, n0 + tx * 4 + j, acc[i][j]);
        return;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
        *reinterpret_cast<float4*>(&Ps[ty * 4 + i][tx * 4]) = make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    cg::cluster_group cluster = cg::this_cluster();
    cluster.sync();
    const int rows = BM / split, r0 = part * rows;
    for (int e = tid; e < rows * BN; e += 256) {
        const int mm = r0 + e / BN, nn = e % BN;
        float v = 0.f;
        for (int r = 0; r < split; ++r) v += cluster.map_shared_rank(&Ps[0][0], r)[mm * BN + nn];
        store(m0 + mm, n0 + nn, v);
    }
    cluster.sync();                                     // partial tiles stay alive until all have read them
}


// ---------------------------------------------------------------------------
// Network layers on the tcgen05 tensor cores (inference).  A layer is
//     C (n x fo) = X Wᵀ,  then + b and GELU (all but the last layer),
// with X held as split BF16 rows [x_hi | x_lo] (x ≈ x_hi + x_lo, K' = 2 kp, kp = fi rounded
// up to 64) and W packed as [W | W] (fo x K', zeros past fi), so one BF16 GEMM over K' gives
// x_hi W + x_lo W in FP32 accumulators: the activations keep ~16 bits beyond BF16 and the
// weights are the BF16 copy the SIMT layers read too.  The kernel is the linear model's
// persistent tcgen05 structure (TMA ring of 128B-swizzled K-major tiles, one thread issuing
// tcgen05.mma into one of two TMEM accumulators, four epilogue warps reading the other with
// tcgen05.ld); the epilogue adds the bias, applies GELU and writes the next layer's split
// BF16 input directly, plus the FP32 pre-activation Z and output Y where asked.
constexpr int kMlpThreads = 192;

template <int BN>
struct MlpTc {
    static constexpr uint32_t B_BYTES = BN * TC_BK * 2;
    static constexpr uint32_t STAGE = TC_A_BYTES + B_BYTES;
    static constexpr uint32_t SMEM = TC_STAGES * STAGE + 1024 + 256;
};

template <int BN>
__global__ void __launch_bounds__(kMlpThreads, 1)
mlp_layer_tc_kernel(const __grid_constant__ CUtensorMap map_x,   // n  x K' split BF16 activations
                    const __grid_constant__ CUtensorMap map_w,   // fo x K' packed BF16 weights
                    int n, int fo, int kblocks, int mtiles, int ntiles, const float* __restrict__ bias,
                    int gelu_on, float* __restrict__ Z, float* __restrict__ Y,
                    __nv_bfloat16* __restrict__ xnext, int kp_next, uint32_t* __restrict__ flags) {
    constexpr uint32_t STAGE = MlpTc<BN>::STAGE;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_addr(smem_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;
    uint8_t* gbase = smem_raw + (base - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + TC_STAGES * STAGE);
    uint64_t* full = bars;
    uint64_t* empty = bars + TC_STAGES;
    uint64_t* tfull = bars + 2 * TC_STAGES;
    uint64_t* tempty = bars + 2 * TC_STAGES + 2;
    uint64_t* drain = bars + 2 * TC_STAGES + 4;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = mtiles * ntiles;
    if (threadIdx.x == 0) {
        for (int st = 0; st < TC_STAGES; ++st) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], 1);
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
                     ::"r"(smem_addr(&s_tmem)), "r"(2 * BN) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;
    auto aborted = [&]() { return *(volatile int*)&s_abort != 0; };

    int issued = 0;
    if (warp == 0 && lane == 0) {
        for (int t = blockIdx.x; t < total && !aborted(); t += gridDim.x) {
            const int mt = t % mtiles, nt = t / mtiles;
            for (int kb = 0; kb < kblocks; ++kb, ++issued) {
                const int st = issued % TC_STAGES;
                if (issued >= TC_STAGES &&
                    !mbar_wait_bounded(&empty[st], (uint32_t)((issued / TC_STAGES) - 1) & 1u, TC_WAIT)) {
                    atomicExch(&s_abort, 1);
                    break;
                }
                if (aborted()) break;
                const uint32_t sa = base + st * STAGE;
                mbar_arrive_expect_tx(&full[st], STAGE);
                tma_load_2d(sa, &map_x, kb * TC_BK, mt * TC_BM, smem_addr(&full[st]));
                tma_load_2d(sa + TC_A_BYTES, &map_w, kb * TC_BK, nt * BN, smem_addr(&full[st]));
            }
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16(TC_BM, BN);
        int it = 0, local = 0;
        for (int t = blockIdx.x; t < total && !aborted(); t += gridDim.x, ++local) {
            const int b = local & 1;
            if (local >= 2 && !mbar_wait_bounded(&tempty[b], (uint32_t)((local >> 1) - 1) & 1u, TC_WAIT)) {
                atomicExch(&s_abort, 1);
                break;
            }
            tc_fence_after();
            const uint32_t acc_addr = tmem + (uint32_t)(b * BN);
            bool ok = true;
            for (int kb = 0; kb < kblocks; ++kb, ++it) {
                const int st = it % TC_STAGES;
                if (!mbar_wait_bounded(&full[st], (uint32_t)(it / TC_STAGES) & 1u, TC_WAIT)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = base + st * STAGE;
                const uint64_t adesc = sw128_desc(sa), bdesc = sw128_desc(sa + TC_A_BYTES);
#pragma unroll
                for (int k = 0; k < TC_BK / 16; ++k)
                    mma_bf16(acc_addr, adesc + 2 * k, bdesc + 2 * k, idesc, (kb > 0 || k > 0) ? 1u : 0u);
                mma_commit(smem_addr(&empty[st]));
            }
            if (!ok) {
                atomicExch(&s_abort, 1);
                break;
            }
            mma_commit(smem_addr(&tfull[b]));
        }
        mma_commit(smem_addr(drain));
    } else if (warp >= 2) {
        // epilogue: thread = row of the tile (TMEM lane quarter of this warp)
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
            const int mt = t % mtiles, nt = t / mtiles;
            const int n0 = nt * BN;
            const int row = mt * TC_BM + quarter * 32 + lane;
            const bool live = row < n;
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32) {
                uint32_t r[32];
                tmem_ld32_nowait(tmem + lane_base + (uint32_t)(b * BN + c0), r);
                const float bl = __ldg(bias + n0 + c0 + lane);        // fo is a multiple of BN
                tmem_wait_ld();
                float z[32], y[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    z[i] = __uint_as_float(r[i]) + __shfl_sync(0xffffffffu, bl, i);
                    y[i] = gelu_on ? gelu(z[i]) : z[i];
                }
                if (!live) continue;
                const size_t o = (size_t)row * fo + n0 + c0;
                if (Z) {
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        *reinterpret_cast<float4*>(Z + o + i) = make_float4(z[i], z[i + 1], z[i + 2], z[i + 3]);
                }
                if (Y) {
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        *reinterpret_cast<float4*>(Y + o + i) = make_float4(y[i], y[i + 1], y[i + 2], y[i + 3]);
                }
                if (xnext) {
                    __nv_bfloat16* hi = xnext + (size_t)row * (2 * kp_next) + n0 + c0;
                    __nv_bfloat16* lo = hi + kp_next;
#pragma unroll
                    for (int i = 0; i < 32; i += 8) {
                        __align__(16) __nv_bfloat16 h8[8], l8[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            h8[q] = __float2bfloat16_rn(y[i + q]);
                            l8[q] = __float2bfloat16_rn(y[i + q] - __bfloat162float(h8[q]));
                        }
                        *reinterpret_cast<uint4*>(hi + i) = *reinterpret_cast<const uint4*>(h8);
                        *reinterpret_cast<uint4*>(lo + i) = *reinterpret_cast<const uint4*>(l8);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[b]);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && aborted()) raise_flag(flags, DEV_ERR_TIMEOUT);
    if (warp == 0 && lane == 0 && aborted()) {
        for (int k = (issued > TC_STAGES ? issued - TC_STAGES : 0); k < issued; ++k)
            mbar_wait_bounded(&full[k % TC_STAGES], (uint32_t)(k / TC_STAGES) & 1u, TC_WAIT);
    }
    if (warp == 1) mbar_wait_bounded(drain, 0, TC_WAIT);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
    }
}

// x (n x fi FP32) -> split BF16 rows [x_hi | 0 .. | x_lo | 0 ..] of width 2 kp
__global__ void split_rows_kernel(const float* __restrict__ x, int n, int fi, int kp,
                                  __nv_bfloat16* __restrict__ xs) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)n * kp) return;
    const int r = (int)(e / kp), k = (int)(e % kp);
    const float v = (k < fi) ? x[(size_t)r * fi + k] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    xs[(size_t)r * 2 * kp + k] = h;
    xs[(size_t)r * 2 * kp + kp + k] = __float2bfloat16_rn(v - __bfloat162float(h));
}

// W (fo x fi BF16) -> [W | W] of width 2 kp, zeros past fi
__global__ void pack_weights_kernel(const __nv_bfloat16* __restrict__ w, int fo, int fi, int kp,
                                    __nv_bfloat16* __restrict__ out) {
    const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long)fo * kp) return;
    const int o = (int)(e / kp), k = (int)(e % kp);
    const __nv_bfloat16 v = (k < fi) ? w[(size_t)o * fi + k] : __float2bfloat16_rn(0.f);
    out[(size_t)o * 2 * kp + k] = v;
    out[(size_t)o * 2 * kp + kp + k] = v;
}

// θ (FP64, N x p) -> x = 2 (θ - lo)/(hi - lo) - 1 (FP32); optional index list
__global__ void normalize_kernel(const double* __restrict__ theta, int n, int p,
                                 const double* __restrict__ lo, const double* __restrict__ hi,
                                 float* __restrict__ x) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * p) return;
    const int j = e % p;
    x[e] = (float)(2.0 * (theta[e] - lo[j]) / (hi[j] - lo[j]) - 1.0);
}

// dZ = dY ⊙ GELU'(Z)
__global__ void gelu_back_kernel(long n, const float* __restrict__ Z, float* __restrict__ dY) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) dY[e] *= gelu_grad(Z[e]);
}

// db[j] = Σ_i dZ[i, j] (fixed order: one thread per column, strided rows)
__global__ void colsum_kernel(int rows, int cols, const float* __restrict__ dZ, float* __restrict__ db) {
    __shared__ float part[256];
    const int j = blockIdx.x;
    float s = 0.f;
    for (int i = threadIdx.x; i < rows; i += blockDim.x) s += dZ[(long)i * cols + j];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) db[j] = part[0];
}

// mean-squared error: dY = (out - y)/n, per-row squared error for the loss
__global__ void mse_kernel(int n, int k, const float* __restrict__ out, const float* __restrict__ y,
                           float* __restrict__ dY, float* __restrict__ row_loss) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float s = 0.f;
    for (int j = 0; j < k; ++j) {
        const float d = out[(long)i * k + j] - y[(long)i * k + j];
        dY[(long)i * k + j] = d / (float)n;
        s = fmaf(d, d, s);
    }
    if (row_loss) row_loss[i] = 0.5f * s;
}

// Adam with bias correction (Kingma & Ba 2015); refreshes the BF16 weight copy
__global__ void adam_kernel(long count, float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                            float eps, float c1, float c2, __nv_bfloat16* __restrict__ pbf) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= count) return;
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi;
    const float vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    const float w = p[e] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[e] = w;
    if (pbf) pbf[e] = __float2bfloat16_rn(w);
}

__global__ void to_bf16_kernel(long count, const float* __restrict__ p, __nv_bfloat16* __restrict__ q) {
    long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < count) q[e] = __float2bfloat16_rn(p[e]);
}

// llk_s = norm - ½ (q0 - 2 hᵀ c̃ + c̃ᵀ G c̃), c̃ = scale ⊙ c ; one warp per chain.  Each CTA
// stages Gᵀ in shared memory once (lane a then reads column a of a row of Gᵀ: consecutive
// words, no bank conflict) and walks chains with a grid stride; the warp's c̃ goes through
// shared memory and is read as a broadcast.
constexpr int kSurMaxK = 96;
constexpr int kSurWarps = 8;
__global__ void __launch_bounds__(kSurWarps * 32)
surrogate_llk_kernel(int n, int k, const float* __restrict__ coeff, const float* __restrict__ scale,
                     const float* __restrict__ G, const float* __restrict__ h, double q0, double norm,
                     double* __restrict__ llk) {
    extern __shared__ float s_mem[];
    float* sGT = s_mem;                                  // k x k, sGT[b k + a] = G[a k + b]
    float* sc = s_mem + k * k + (threadIdx.x >> 5) * k;  // this warp's c̃
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int a = e / k, b = e - a * k;
        sGT[b * k + a] = G[e];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * kSurWarps;
    for (int i = blockIdx.x * kSurWarps + (threadIdx.x >> 5); i < n; i += stride) {
        const float* c = coeff + (long)i * k;
        for (int b = lane; b < k; b += 32) sc[b] = c[b] * scale[b];
        __syncwarp();
        double acc = 0.0;
        for (int a = lane; a < k; a += 32) {
            const float ca = sc[a];
            float row = 0.f;
            for (int b = 0; b < k; ++b) row = fmaf(sGT[b * k + a], sc[b], row);
            acc += (double)ca * (double)row - 2.0 * (double)h[a] * (double)ca;
        }
        acc = warp_sum(acc);
        if (lane == 0) llk[i] = norm - 0.5 * (q0 + acc);
        __syncwarp();
    }
}

// Stage 1 of delayed acceptance: surrogate Metropolis test and compaction of survivors
__global__ void da_screen_kernel(int n, const double* __restrict__ beta, uint64_t seed, uint32_t step,
                                 const uint32_t* __restrict__ epoch, const uint32_t* __restrict__ mask,
                                 const double* __restrict__ cprior, const double* __restrict__ csur,
                                 const double* __restrict__ prior, const double* __restrict__ sur,
                                 int32_t* __restrict__ pass, int32_t* __restrict__ index,
                                 int32_t* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int ok = 0;
    if (!mask[i]) {
        const double b = *beta;
        const double d1 = (cprior[i] + b * csur[i]) - (prior[i] + b * sur[i]);
        u32x4 r = draw(seed, (uint32_t)i, 1u, STREAM_ACCEPT, step, *epoch);
        ok = log(u01_open_closed(r.x, r.y)) <= d1;
    }
    pass[i] = ok;
    if (ok) index[atomicAdd(count, 1)] = i;
}

// Stage 2: exact correction for the survivors; counters: accepted, rejected (support), unlikely
__global__ void da_accept_kernel(int n, int p, const double* __restrict__ beta, uint64_t seed,
                                 uint32_t step, const uint32_t* __restrict__ epoch,
                                 const uint32_t* __restrict__ mask, const int32_t* __restrict__ pass,
                                 const double* __restrict__ cand, const double* __restrict__ cprior,
                                 const double* __restrict__ cdata, const double* __restrict__ csur,
                                 double* __restrict__ theta, double* __restrict__ prior,
                                 double* __restrict__ data, double* __restrict__ post,
                                 double* __restrict__ sur, unsigned long long* __restrict__ counters,
                                 unsigned long long* __restrict__ screened) {
    __shared__ unsigned int s_cnt[4];
    if (threadIdx.x < 4) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if (mask[i]) {
            atomicAdd(&s_cnt[1], 1u);
        } else if (!pass[i]) {
            atomicAdd(&s_cnt[2], 1u);
        } else {
            atomicAdd(&s_cnt[3], 1u);
            const double b = *beta;
            const double cp = cprior[i] + b * cdata[i];
            const double dsur = (cprior[i] + b * csur[i]) - (prior[i] + b * sur[i]);
            u32x4 r = draw(seed, (uint32_t)i, 2u, STREAM_ACCEPT, step, *epoch);
            if (log(u01_open_closed(r.x, r.y)) > (cp - post[i]) - dsur) {
                atomicAdd(&s_cnt[2], 1u);
            } else {
                atomicAdd(&s_cnt[0], 1u);
                for (int j = 0; j < p; ++j) theta[(size_t)i * p + j] = cand[(size_t)i * p + j];
                prior[i] = cprior[i];
                data[i] = cdata[i];
                post[i] = cp;
                sur[i] = csur[i];
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < 3 && s_cnt[threadIdx.x])
        atomicAdd(&counters[threadIdx.x], (unsigned long long)s_cnt[threadIdx.x]);
    if (threadIdx.x == 3 && s_cnt[3] && screened) atomicAdd(screened, (unsigned long long)s_cnt[3]);
}

// The exact log-likelihood below which the stage-2 test of da_accept_kernel certainly
// rejects chain i (early rejection of the exact correction): the test rejects when
// log u > (cprior + β cdata − post) − dsur, so below (log u + post − cprior + dsur)/β, lowered
// by a relative 1e-9 for the rounding of the test; -inf where no evaluation is made.
__global__ void da_floor_kernel(int n, const double* __restrict__ beta, uint64_t seed, uint32_t step,
                                const uint32_t* __restrict__ epoch, const uint32_t* __restrict__ mask,
                                const int32_t* __restrict__ pass, const double* __restrict__ cprior,
                                const double* __restrict__ csur, const double* __restrict__ prior,
                                const double* __restrict__ sur, const double* __restrict__ post,
                                double* __restrict__ floor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double b = *beta;
    double f = -INFINITY;
    if (!mask[i] && pass[i] && b > 0.0) {
        const double dsur = (cprior[i] + b * csur[i]) - (prior[i] + b * sur[i]);
        u32x4 r = draw(seed, (uint32_t)i, 2u, STREAM_ACCEPT, step, *epoch);
        f = (log(u01_open_closed(r.x, r.y)) + post[i] - cprior[i] + dsur) / b;
        f -= (fabs(f) + 1.0) * 1e-9;
        if (!(f == f)) f = -INFINITY;
    }
    floor[i] = f;
}

// chains whose surrogate-chain state moved away from the exact state go to the exact
// correction: pass[i] = (θ_s ≠ θ) and no support violation, compacted into index
__global__ void da_moved_kernel(int n, int p, const double* __restrict__ theta,
                                const double* __restrict__ theta_s, int32_t* __restrict__ pass,
                                int32_t* __restrict__ index, int32_t* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int moved = 0;
    for (int j = 0; j < p; ++j) moved |= (theta[(size_t)i * p + j] != theta_s[(size_t)i * p + j]);
    pass[i] = moved;
    if (moved) index[atomicAdd(count, 1)] = i;
}

}  // namespace ag

// ---------------------------------------------------------------------------
// C ABI
using namespace ag;

static inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

extern "C" int ag_da_moved(int32_t n, int32_t p, const double* theta, const double* theta_s, int32_t* pass,
                           int32_t* index, int32_t* count, void* stream) {
    AG_REQUIRE(n > 0 && p > 0 && theta && theta_s && pass && index && count, "invalid arguments");
    cudaStream_t s = as_stream(stream);
    int rc = cuda_status(cudaMemsetAsync(count, 0, sizeof(int32_t), s), "memset count");
    if (rc) return rc;
    da_moved_kernel<<<nblk(n, 256), 256, 0, s>>>(n, p, theta, theta_s, pass, index, count);
    return launch_status("da_moved_kernel");
}

static int check_net(const ag_mlp* net) {
    AG_REQUIRE(net && net->nlayers >= 1 && net->nlayers <= kMaxLayers, "invalid network");
    for (int l = 0; l <= net->nlayers; ++l) AG_REQUIRE(net->sizes[l] > 0, "layer size must be positive");
    return AG_OK;
}

extern "C" int64_t ag_mlp_param_count(const ag_mlp* net) {
    if (check_net(net)) return -1;
    int64_t c = 0;
    for (int l = 0; l < net->nlayers; ++l) c += (int64_t)net->sizes[l + 1] * net->sizes[l] + net->sizes[l + 1];
    return c;
}

// parameter layout: for each layer W (out x in) then b (out)
static void offsets(const ag_mlp* net, int64_t* w, int64_t* b) {
    int64_t c = 0;
    for (int l = 0; l < net->nlayers; ++l) {
        w[l] = c;
        c += (int64_t)net->sizes[l + 1] * net->sizes[l];
        b[l] = c;
        c += net->sizes[l + 1];
    }
}

extern "C" int64_t ag_mlp_activation_floats(const ag_mlp* net, int32_t n) {
    if (check_net(net) || n <= 0) return -1;
    int64_t c = 0;
    for (int l = 1; l <= net->nlayers; ++l) c += 2 * (int64_t)n * net->sizes[l];   // Z and Y per layer
    return c;
}

// Split K over a cluster of up to 8 CTAs when the output tiles alone would leave most of the
// GPU idle (the weight gradients: a few tiles, K = batch rows).
static int gemm(cudaStream_t s, int M, int N, int K, const float* A, long sam, long sak, const void* B,
                bool bbf16, long sbk, long sbn, float* C, long ldc, const float* bias, int epi, float* Z) {
    const int tiles = nblk(N, BN) * nblk(M, BM);
    int split = 1;
    while (split < 8 && tiles * split < 128 && K >= 2 * BK * (split * 2)) split *= 2;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nblk(N, BN), nblk(M, BM), split);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 1;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = split;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = bbf16 ? cudaLaunchKernelEx(&cfg, gemm_kernel<true>, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc,
                                               bias, epi, Z)
                          : cudaLaunchKernelEx(&cfg, gemm_kernel<false>, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc,
                                               bias, epi, Z);
    int rc = cuda_status(e, "cudaLaunchKernelEx(gemm_kernel)");
    if (rc) return rc;
    return launch_status("gemm_kernel");
}

extern "C" int ag_normalize_inputs(const double* theta, int32_t n, int32_t p, const double* lo,
                                   const double* hi, float* x, void* stream) {
    AG_REQUIRE(theta && lo && hi && x && n > 0 && p > 0, "invalid arguments");
    normalize_kernel<<<nblk((long)n * p, 256), 256, 0, as_stream(stream)>>>(theta, n, p, lo, hi, x);
    return launch_status("normalize_kernel");
}

extern "C" int ag_mlp_forward(const ag_mlp* net, const float* params, const uint16_t* wbf16,
                              const float* x, int32_t n, float* out, float* acts, void* stream) {
    int rc = check_net(net);
    if (rc) return rc;
    AG_REQUIRE(params && wbf16 && x && out && acts && n > 0, "invalid arguments");
    cudaStream_t s = as_stream(stream);
    int64_t wo[kMaxLayers], bo[kMaxLayers];
    offsets(net, wo, bo);
    const float* in = x;
    float* a = acts;
    for (int l = 0; l < net->nlayers; ++l) {
        const int fi = net->sizes[l], fo = net->sizes[l + 1];
        const bool last = (l == net->nlayers - 1);
        float* Z = a;
        float* Y = last ? out : a + (int64_t)n * fo;
        rc = gemm(s, n, fo, fi, in, fi, 1, wbf16 + wo[l], true, 1, fi, Y, fo, params + bo[l],
                  last ? EPI_BIAS : EPI_BIAS_GELU, Z);
        if (rc) return rc;
        in = Y;
        a += 2 * (int64_t)n * fo;
    }
    return AG_OK;
}

// ---- tensor-core forward (inference)
static int mlp_kp(int f) { return (f + 63) / 64 * 64; }

static int check_net_tc(const ag_mlp* net) {
    int rc = check_net(net);
    if (rc) return rc;
    for (int l = 1; l <= net->nlayers; ++l)
        AG_REQUIRE(net->sizes[l] % 64 == 0, "the tensor-core layers need widths that are multiples of 64 "
                                            "(layer %d has %d)", l, net->sizes[l]);
    return AG_OK;
}

extern "C" size_t ag_mlp_tc_pack_bytes(const ag_mlp* net) {
    if (check_net_tc(net)) return 0;
    size_t c = 0;
    for (int l = 0; l < net->nlayers; ++l) c += (size_t)net->sizes[l + 1] * 2 * mlp_kp(net->sizes[l]) * 2;
    return c;
}

extern "C" int ag_mlp_tc_pack(const ag_mlp* net, const uint16_t* wbf16, uint16_t* wpack, void* stream) {
    int rc = check_net_tc(net);
    if (rc) return rc;
    AG_REQUIRE(wbf16 && wpack && aligned(wpack, 256), "invalid arguments (wpack must be 256-byte aligned)");
    cudaStream_t s = as_stream(stream);
    int64_t wo[kMaxLayers], bo[kMaxLayers];
    offsets(net, wo, bo);
    size_t off = 0;
    for (int l = 0; l < net->nlayers; ++l) {
        const int fi = net->sizes[l], fo = net->sizes[l + 1], kp = mlp_kp(fi);
        pack_weights_kernel<<<nblk((long)fo * kp, 256), 256, 0, s>>>(
            reinterpret_cast<const __nv_bfloat16*>(wbf16) + wo[l], fo, fi, kp,
            reinterpret_cast<__nv_bfloat16*>(wpack) + off);
        rc = launch_status("pack_weights_kernel");
        if (rc) return rc;
        off += (size_t)fo * 2 * kp;
    }
    return AG_OK;
}

extern "C" size_t ag_mlp_tc_workspace_bytes(const ag_mlp* net, int32_t n) {
    if (check_net_tc(net) || n <= 0) return 0;
    int kmax = 0;
    for (int l = 0; l < net->nlayers; ++l) kmax = max(kmax, mlp_kp(net->sizes[l]));
    const size_t one = ((size_t)n * 2 * kmax * 2 + 255) / 256 * 256;
    return 2 * one;
}

template <int BN>
static int mlp_layer_launch(cudaStream_t s, const __nv_bfloat16* xs, int n, int kp, const __nv_bfloat16* w,
                            int fo, const float* bias, int gelu_on, float* Z, float* Y, __nv_bfloat16* xnext,
                            int kp_next, uint32_t* flags) {
    CUtensorMap mx, mw;
    int rc = make_map(&mx, xs, n, 2 * kp, TC_BM);
    if (rc) return rc;
    rc = make_map(&mw, w, fo, 2 * kp, BN);
    if (rc) return rc;
    rc = cuda_status(cudaFuncSetAttribute(mlp_layer_tc_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)MlpTc<BN>::SMEM),
                     "cudaFuncSetAttribute(mlp_layer_tc_kernel)");
    if (rc) return rc;
    int sms = 0;
    rc = sm_count(&sms);
    if (rc) return rc;
    const int mtiles = (n + TC_BM - 1) / TC_BM, ntiles = fo / BN, total = mtiles * ntiles;
    mlp_layer_tc_kernel<BN><<<total < sms ? total : sms, kMlpThreads, MlpTc<BN>::SMEM, s>>>(
        mx, mw, n, fo, 2 * kp / TC_BK, mtiles, ntiles, bias, gelu_on, Z, Y, xnext, kp_next, flags);
    return launch_status("mlp_layer_tc_kernel");
}

extern "C" int ag_mlp_forward_tc(const ag_mlp* net, const float* params, const uint16_t* wpack, const float* x,
                                 int32_t n, float* out, float* acts, void* workspace, size_t workspace_bytes,
                                 uint32_t* flags, void* stream) {
    int rc = check_net_tc(net);
    if (rc) return rc;
    AG_REQUIRE(params && wpack && x && out && flags && n > 0, "invalid arguments");
    AG_REQUIRE(aligned(out, 16) && (acts == nullptr || aligned(acts, 16)) && aligned(wpack, 256),
               "out and acts must be 16-byte aligned, wpack 256-byte aligned");
    const size_t need = ag_mlp_tc_workspace_bytes(net, n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "the tensor-core forward needs %zu bytes of 256-byte aligned workspace", need);
    cudaStream_t s = as_stream(stream);
    int64_t wo[kMaxLayers], bo[kMaxLayers];
    offsets(net, wo, bo);
    __nv_bfloat16* buf[2] = {reinterpret_cast<__nv_bfloat16*>(workspace),
                             reinterpret_cast<__nv_bfloat16*>(static_cast<char*>(workspace) + need / 2)};
    const int fi0 = net->sizes[0], kp0 = mlp_kp(fi0);
    split_rows_kernel<<<nblk((long)n * kp0, 256), 256, 0, s>>>(x, n, fi0, kp0, buf[0]);
    rc = launch_status("split_rows_kernel");
    if (rc) return rc;
    const __nv_bfloat16* w = reinterpret_cast<const __nv_bfloat16*>(wpack);
    float* a = acts;
    for (int l = 0; l < net->nlayers; ++l) {
        const int fi = net->sizes[l], fo = net->sizes[l + 1], kp = mlp_kp(fi);
        const bool last = (l == net->nlayers - 1);
        float* Z = (a && !last) ? a : nullptr;
        float* Y = last ? out : (a ? a + (int64_t)n * fo : nullptr);
        __nv_bfloat16* xnext = last ? nullptr : buf[(l + 1) & 1];
        const int kp_next = last ? 0 : mlp_kp(fo);
        rc = (fo % 256 == 0)
                 ? mlp_layer_launch<256>(s, buf[l & 1], n, kp, w, fo, params + bo[l], last ? 0 : 1, Z, Y, xnext,
                                         kp_next, flags)
                 : mlp_layer_launch<64>(s, buf[l & 1], n, kp, w, fo, params + bo[l], last ? 0 : 1, Z, Y, xnext,
                                        kp_next, flags);
        if (rc) return rc;
        w += (size_t)fo * 2 * kp;
        if (a) a += 2 * (int64_t)n * fo;
    }
    return AG_OK;
}

extern "C" int ag_mlp_backward(const ag_mlp* net, const float* params, const uint16_t* wbf16,
                               const float* x, int32_t n, const float* acts, float* dout, float* grads,
                               float* scratch, void* stream) {
    int rc = check_net(net);
    if (rc) return rc;
    AG_REQUIRE(params && wbf16 && x && acts && dout && grads && scratch && n > 0, "invalid arguments");
    cudaStream_t s = as_stream(stream);
    int64_t wo[kMaxLayers], bo[kMaxLayers], ao[kMaxLayers];
    offsets(net, wo, bo);
    int64_t c = 0;
    int maxw = 0;
    for (int l = 0; l < net->nlayers; ++l) {
        ao[l] = c;
        c += 2 * (int64_t)n * net->sizes[l + 1];
        maxw = max(maxw, net->sizes[l + 1]);
        maxw = max(maxw, net->sizes[l]);
    }
    // dY of the current layer lives in dout (last layer) or in scratch (n x maxw, ping-pong)
    float* cur = dout;
    float* bufs[2] = {scratch, scratch + (int64_t)n * maxw};
    for (int l = net->nlayers - 1; l >= 0; --l) {
        const int fi = net->sizes[l], fo = net->sizes[l + 1];
        const bool last = (l == net->nlayers - 1);
        if (!last) {
            gelu_back_kernel<<<nblk((long)n * fo, 256), 256, 0, s>>>((long)n * fo, acts + ao[l], cur);
            rc = launch_status("gelu_back_kernel");
            if (rc) return rc;
        }
        const float* hin = (l == 0) ? x : acts + ao[l - 1] + (int64_t)n * fi;   // Y of layer l-1
        // dW (fo x fi) = dZᵀ (fo x n) · h (n x fi)
        rc = gemm(s, fo, fi, n, cur, 1, fo, hin, false, fi, 1, grads + wo[l], fi, nullptr, EPI_NONE, nullptr);
        if (rc) return rc;
        colsum_kernel<<<fo, 256, 0, s>>>(n, fo, cur, grads + bo[l]);
        rc = launch_status("colsum_kernel");
        if (rc) return rc;
        if (l > 0) {
            float* nxt = bufs[l & 1];
            // dX (n x fi) = dZ (n x fo) · W (fo x fi)
            rc = gemm(s, n, fi, fo, cur, fo, 1, wbf16 + wo[l], true, fi, 1, nxt, fi, nullptr, EPI_NONE, nullptr);
            if (rc) return rc;
            cur = nxt;
        }
    }
    return AG_OK;
}

extern "C" int ag_mse_grad(int32_t n, int32_t k, const float* out, const float* target, float* dout,
                           float* row_loss, void* stream) {
    AG_REQUIRE(n > 0 && k > 0 && out && target && dout, "invalid arguments");
    mse_kernel<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(n, k, out, target, dout, row_loss);
    return launch_status("mse_kernel");
}

extern "C" int ag_adam_step(int64_t count, float* params, const float* grads, float* m, float* v,
                            int32_t t, float lr, float b1, float b2, float eps, uint16_t* wbf16,
                            void* stream) {
    AG_REQUIRE(count > 0 && params && grads && m && v && t >= 1, "invalid arguments");
    const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
    adam_kernel<<<nblk(count, 256), 256, 0, as_stream(stream)>>>(
        count, params, grads, m, v, lr, b1, b2, eps, c1, c2, reinterpret_cast<__nv_bfloat16*>(wbf16));
    return launch_status("adam_kernel");
}

extern "C" int ag_to_bf16(int64_t count, const float* src, uint16_t* dst, void* stream) {
    AG_REQUIRE(count > 0 && src && dst, "invalid arguments");
    to_bf16_kernel<<<nblk(count, 256), 256, 0, as_stream(stream)>>>(count, src,
                                                                     reinterpret_cast<__nv_bfloat16*>(dst));
    return launch_status("to_bf16_kernel");
}

extern "C" int ag_surrogate_llk(int32_t n, int32_t k, const float* coeff, const float* scale,
                                const float* gram, const float* h, double q0, double norm, double* llk,
                                void* stream) {
    AG_REQUIRE(n > 0 && k > 0 && coeff && scale && gram && h && llk, "invalid arguments");
    AG_REQUIRE(k <= kSurMaxK, "at most %d surrogate coefficients are supported (got %d)", kSurMaxK, k);
    const size_t smem = (size_t)(k * k + kSurWarps * k) * sizeof(float);
    int dev = 0, sms = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "multiProcessorCount");
    if (rc) return rc;
    const int grid = min(nblk(n, kSurWarps), 4 * sms);
    surrogate_llk_kernel<<<grid, kSurWarps * 32, smem, as_stream(stream)>>>(n, k, coeff, scale, gram, h, q0,
                                                                           norm, llk);
    return launch_status("surrogate_llk_kernel");
}

extern "C" int ag_da_screen(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step,
                            const uint32_t* mask, const double* cprior, const double* csur,
                            const double* prior, const double* sur, int32_t* pass, int32_t* index,
                            int32_t* count, void* stream) {
    AG_REQUIRE(st && n > 0 && mask && cprior && csur && prior && sur && pass && index && count,
               "invalid arguments");
    cudaStream_t s = as_stream(stream);
    int rc = cuda_status(cudaMemsetAsync(count, 0, sizeof(int32_t), s), "memset count");
    if (rc) return rc;
    da_screen_kernel<<<nblk(n, 256), 256, 0, s>>>(n, st->beta, seed, step, st->epoch, mask, cprior, csur,
                                                  prior, sur, pass, index, count);
    return launch_status("da_screen_kernel");
}

extern "C" int ag_da_floor(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step, const uint32_t* mask,
                           const int32_t* pass, const double* cprior, const double* csur, const double* prior,
                           const double* sur, const double* post, double* llk_floor, void* stream) {
    AG_REQUIRE(st && n > 0 && mask && pass && cprior && csur && prior && sur && post && llk_floor,
               "invalid arguments");
    da_floor_kernel<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(n, st->beta, seed, step, st->epoch, mask, pass,
                                                                  cprior, csur, prior, sur, post, llk_floor);
    return launch_status("da_floor_kernel");
}

extern "C" int ag_da_accept(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed, uint32_t step,
                            const uint32_t* mask, const int32_t* pass, const double* cand,
                            const double* cprior, const double* cdata, const double* csur, double* theta,
                            double* prior, double* data, double* post, double* sur,
                            unsigned long long* screened, void* stream) {
    AG_REQUIRE(st && n > 0 && p > 0 && mask && pass && cand && cprior && cdata && csur && theta && prior &&
                   data && post && sur,
               "invalid arguments");
    da_accept_kernel<<<nblk(n, 256), 256, 0, as_stream(stream)>>>(
        n, p, st->beta, seed, step, st->epoch, mask, pass, cand, cprior, cdata, csur, theta, prior, data,
        post, sur, st->counters, screened);
    return launch_status("da_accept_kernel");
}
