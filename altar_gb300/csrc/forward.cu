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
// constants and per-rectangle quadrature parameters in FP64 and packs the
// chains that have work (not masked, not above the free surface) into
// consecutive slots; the likelihood kernel runs one warp per slot, lanes over
// stations; a CTA holds WARPS chains whose constants live in shared memory and
// are read with broadcast vector loads; station tiles stream through a ring of
// shared-memory buffers filled by 1-D bulk copies (cp.async.bulk + mbarrier)
// and shared by the CTA's warps.  For each tile a warp decides, from the
// tile's bounding box, which rectangles it integrates by quadrature and with
// how many nodes (generated into shared memory), and evaluates the sides of the
// others.  Each lane accumulates w·r² in float-float; the warp's sum is reduced
// in FP64 in a fixed order.
#include <math.h>
#include <stdint.h>

#include "common.cuh"
#include "internal.h"
#include "cdm_side.cuh"

namespace ag {

constexpr int kMaxOffsets = 16;      // datasets with their own offset parameter
constexpr int kTile = AG_STATION_TILE;
constexpr uint32_t kWaitLimit = 1u << 24;

// ---------------------------------------------------------------------------
// per-chain constants: stations are taken relative to the source centre (x0, y0)
struct __align__(16) ChainC {
    float4 hdr;                 // x0_hi, x0_lo, y0_hi, y0_lo
    uint32_t side_mask;         // active sides; 0 = chain inactive
    uint32_t status;
    uint32_t pad0, pad1;
    float off[kMaxOffsets];     // per-dataset offsets θ[offset_idx + k]
    float pad2[8];
    SideC side[kSides];
    RectQ rect[3];              // every rectangle that takes part, parametric quadrature
};
static_assert(sizeof(ChainC) % 16 == 0, "ChainC must be a whole number of float4");

// Chain slots ordered by cost.  The chains of one CTA share its ring of station tiles, so a
// CTA advances at the pace of its most expensive chain; with rectangles integrated by
// quadrature, with node counts that depend on each tile's distance, the work of a chain
// ranges over several times its minimum.  The set-up therefore runs in two passes:
// cdm_cost_kernel classifies every requested chain (masked, above the free surface, or the
// cost bucket of its plan averaged over a sample of the tiles) and counts the chains per
// bucket; cdm_setup_kernel gives each chain the next slot of its bucket, buckets in
// decreasing cost, so the CTAs hold chains of similar cost and the expensive ones are
// scheduled first (which also shortens the tail of the launch for one-chain CTAs).
constexpr int kCostBuckets = 64;
constexpr int kCostBucketFlop = 96;      // FLOP per station per bucket

struct SetupHdr {                        // in the workspace, cleared before each set-up
    int32_t nslots;
    int32_t pad[31];
    int32_t hist[kCostBuckets];          // chains per cost bucket
    int32_t fill[kCostBuckets];          // slots handed out per bucket
};

__device__ __forceinline__ int cost_bucket(uint32_t flop) {
    const int b = (int)(flop / kCostBucketFlop);
    return b < kCostBuckets - 1 ? b : kCostBuckets - 1;
}

// Per-station work of a chain averaged over every stride-th station tile (tile boxes
// relative to the source centre as the likelihood kernel forms them)
__device__ float sampled_tile_work(const RectQ* rect, uint32_t mask, const float4* __restrict__ tile_box,
                                   int ntiles, int stride, float x0h, float x0l, float y0h, float y0l) {
    float f = 0.f;
    int cnt = 0;
    for (int t = stride / 2; t < ntiles; t += stride) {
        const float4 tb = __ldg(tile_box + t);
        uint32_t fl, su;
        tile_work(rect, mask, __fsub_rn(__fsub_rn(tb.x, x0h), x0l), __fsub_rn(__fsub_rn(tb.y, x0h), x0l),
                  __fsub_rn(__fsub_rn(tb.z, y0h), y0l), __fsub_rn(__fsub_rn(tb.w, y0h), y0l), fl, su);
        f += (float)fl;
        ++cnt;
    }
    return cnt ? f / (float)cnt : (float)kFlopStation;
}

// One thread per requested chain (all n, or the first *count_in of index_in): -1 for a masked
// chain, -2 (and the status bit) for one above the free surface, else its cost bucket (the
// work of its plan averaged over a sample of the station tiles)
__global__ void cdm_cost_kernel(ag_layout L, const double* __restrict__ theta, int n,
                                const uint32_t* __restrict__ mask_in, uint32_t* __restrict__ chain_status,
                                const int32_t* __restrict__ index_in, const int32_t* __restrict__ count_in,
                                const float4* __restrict__ tile_box, int ntiles, int8_t* __restrict__ key,
                                SetupHdr* __restrict__ hdr) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i = t;
    if (index_in) {
        if (t >= *count_in) return;
        i = index_in[t];
    }
    if (mask_in && mask_in[i]) {
        key[t] = -1;
        return;
    }
    const double* th = theta + (size_t)i * L.nparams;
    Vec3 V[3][4];
    if (cdm_corners(th, L, V)) {
        if (chain_status) chain_status[i] |= CHAIN_ABOVE_SURFACE;
        key[t] = -2;
        return;
    }
    const double x0 = th[L.x_idx], y0 = th[L.x_idx + 1];
    float x0h, x0l, y0h, y0l;
    split_hilo(x0, x0h, x0l);
    split_hilo(y0, y0h, y0l);
    RectQ rect[3];
    const uint32_t mask = cdm_rects(th, L, V, x0, y0, rect);
    const int stride = ntiles > 16 ? ntiles / 16 : 1;
    const int b = cost_bucket((uint32_t)sampled_tile_work(rect, mask, tile_box, ntiles, stride, x0h, x0l, y0h, y0l));
    key[t] = (int8_t)b;
    atomicAdd(&hdr->hist[b], 1);
}

// Every chain with work takes the next slot of its cost bucket (buckets in decreasing cost;
// the order inside a bucket is that of the atomic, which does not affect any chain's result)
// and writes its constants there, so the likelihood kernel's CTAs hold only chains with work.
__global__ void cdm_setup_kernel(ag_layout L, const double* __restrict__ theta, int n,
                                 const int8_t* __restrict__ key, ChainC* __restrict__ out, int noffsets,
                                 const int32_t* __restrict__ index_in, const int32_t* __restrict__ count_in,
                                 int32_t* __restrict__ index_out, SetupHdr* __restrict__ hdr) {
    __shared__ int s_start[kCostBuckets];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = kCostBuckets - 1; b >= 0; --b) {
            s_start[b] = acc;
            acc += hdr->hist[b];
        }
        if (blockIdx.x == 0) hdr->nslots = acc;
    }
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int i = t;
    if (index_in) {
        if (t >= *count_in) return;
        i = index_in[t];
    }
    const int b = key[t];
    if (b < 0) return;
    const double* th = theta + (size_t)i * L.nparams;
    Vec3 V[3][4];
    cdm_corners(th, L, V);
    const int slot = s_start[b] + atomicAdd(&hdr->fill[b], 1);
    index_out[slot] = i;
    ChainC& C = out[slot];
    C.side_mask = 0u;
    C.status = 0u;
    const double x0 = th[L.x_idx], y0 = th[L.x_idx + 1];
    split_hilo(x0, C.hdr.x, C.hdr.y);
    split_hilo(y0, C.hdr.z, C.hdr.w);
    for (int k = 0; k < kMaxOffsets; ++k)
        C.off[k] = (k < noffsets) ? (float)th[L.offset_idx + k] : 0.f;
    const uint32_t mask = cdm_sides(th, L, V, x0, y0, C.side, C.rect);
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

// FP32 operations the likelihood kernel executes for each chain over the m stations (its
// plan per station tile: sides and quadrature nodes); 0 for chains above the free surface,
// which it skips
__global__ void cdm_work_kernel(ag_layout L, const double* __restrict__ theta, int n,
                                const float4* __restrict__ tile_box, int m, double* __restrict__ flop,
                                double* __restrict__ sfu) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* th = theta + (size_t)i * L.nparams;
    Vec3 V[3][4];
    double f = 0.0, u = 0.0;
    if (!cdm_corners(th, L, V)) {
        const double x0 = th[L.x_idx], y0 = th[L.x_idx + 1];
        float x0h, x0l, y0h, y0l;
        split_hilo(x0, x0h, x0l);
        split_hilo(y0, y0h, y0l);
        RectQ rect[3];
        const uint32_t mask = cdm_rects(th, L, V, x0, y0, rect);
        const int ntiles = (m + kTile - 1) / kTile;
        for (int t = 0; t < ntiles; ++t) {
            const float4 tb = __ldg(tile_box + t);
            uint32_t fl, su;
            tile_work(rect, mask, __fsub_rn(__fsub_rn(tb.x, x0h), x0l), __fsub_rn(__fsub_rn(tb.y, x0h), x0l),
                      __fsub_rn(__fsub_rn(tb.z, y0h), y0l), __fsub_rn(__fsub_rn(tb.w, y0h), y0l), fl, su);
            const int cnt = min(kTile, m - t * kTile);
            f += (double)fl * cnt;
            u += (double)su * cnt;
        }
    }
    flop[i] = f;
    if (sfu) sfu[i] = u;
}

// Bounding box of each tile of AG_STATION_TILE stations (coordinates hi + lo), rounded
// outwards to FP32; padding stations (index >= m) are left out.  One warp per tile.
__global__ void station_boxes_kernel(const float4* __restrict__ xy, int m, int ntiles, float4* __restrict__ box) {
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (t >= ntiles) return;
    double x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
    for (int j = t * kTile + lane; j < min(m, (t + 1) * kTile); j += 32) {
        const float4 a = xy[j];
        const double x = (double)a.x + (double)a.y, y = (double)a.z + (double)a.w;
        x0 = fmin(x0, x); x1 = fmax(x1, x);
        y0 = fmin(y0, y); y1 = fmax(y1, y);
    }
    for (int o = 16; o > 0; o >>= 1) {
        x0 = fmin(x0, __shfl_xor_sync(0xffffffffu, x0, o));
        x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
        y0 = fmin(y0, __shfl_xor_sync(0xffffffffu, y0, o));
        y1 = fmax(y1, __shfl_xor_sync(0xffffffffu, y1, o));
    }
    if (lane == 0) box[t] = make_float4(f32_down(x0), f32_up(x1), f32_down(y0), f32_up(y1));
}

// ---------------------------------------------------------------------------
// CDM likelihood.  One warp per compacted chain slot, lanes over stations.
// Station tiles stream through a ring of STAGES shared-memory buffers filled
// by 1-D bulk copies: each warp waits on the buffer's full barrier, works
// through the tile and counts itself done; the warp that finishes a tile last
// refills that buffer with the tile STAGES ahead.  No CTA-wide barrier is
// taken per tile, so warps drift apart by up to STAGES - 1 tiles instead of
// waiting for the slowest one at every tile.
template <int WARPS, int MINB, int SPL, int STAGES>
__global__ void __launch_bounds__(WARPS * 32, MINB)
cdm_llk_kernel(const ChainC* __restrict__ chains, const int32_t* __restrict__ slot_chain,
               const int32_t* __restrict__ nslots_ptr, int n, const float4* __restrict__ xy,
               const float4* __restrict__ losd, const float* __restrict__ wt,
               const int32_t* __restrict__ oid, const float4* __restrict__ tile_box,
               const int32_t* __restrict__ order, int m, int m_padded, double norm,
               const double* __restrict__ llk_floor, double* __restrict__ llk, float* __restrict__ resid,
               uint32_t* __restrict__ flags) {
    const int nslots = min(n, *nslots_ptr);
    if ((int)(blockIdx.x * WARPS) >= nslots) return;       // whole CTA past the active chains
    __shared__ ChainC s_chain[WARPS];
    __shared__ float4 s_xy[STAGES][kTile];
    __shared__ float4 s_ld[STAGES][kTile];
    __shared__ __align__(16) float s_w[STAGES][kTile];
    __shared__ __align__(16) int32_t s_oid[STAGES][kTile];
    __shared__ float4 s_box[STAGES];                  // each tile's bounding box, with the tile
    __shared__ __align__(8) uint64_t full[STAGES];
    __shared__ int s_done[STAGES];
    __shared__ int s_issued;
    // each warp's quadrature nodes: one buffer per rectangle (one shared by the three where
    // shared memory is short), regenerated only when a tile needs other node counts
    constexpr int kNodeBufs = WARPS <= 4 ? 3 : 1;
    __shared__ float4 s_node[WARPS][kNodeBufs][kQuadBudget];
    __shared__ float s_gx[136], s_gw[136];             // Gauss-Legendre rules (FP32)

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int slot = blockIdx.x * WARPS + warp;
    const bool active = slot < nslots;
    const int chain = active ? slot_chain[slot] : n;
    const int ntiles = m_padded / kTile;
    const bool with_oid = (oid != nullptr);
    const uint32_t tile_bytes = kTile * (16u + 16u + 4u) + (with_oid ? kTile * 4u : 0u) + 16u;

    for (int k = threadIdx.x; k < 136; k += blockDim.x) {
        s_gx[k] = kGaussXf[k];
        s_gw[k] = kGaussWf[k];
    }
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
        bulk_g2s(&s_box[buf], tile_box + t, 16u, &full[buf]);
    };
    if (threadIdx.x == 0) {
        for (int b = 0; b < STAGES; ++b) {
            mbar_init(&full[b], 1);
            s_done[b] = 0;
        }
        fence_mbar_init();
        const int first = ntiles < STAGES ? ntiles : STAGES;
        for (int t = 0; t < first; ++t) issue(t, t);
        s_issued = first;
    }
    __syncthreads();
    const ChainC& C = s_chain[warp];
    const uint32_t smask = active ? C.side_mask : 0u;
    const float x0h = C.hdr.x, x0l = C.hdr.y, y0h = C.hdr.z, y0l = C.hdr.w;
    ff acc{0.f, 0.f};
    bool failed = false;
    uint64_t node_keys = ~0ull;       // 12 bits per buffer: rectangle, n1, n2 of the nodes it holds
    // early rejection: the misfit only grows with the stations, so once the partial
    // log-likelihood is below the chain's floor the proposal is certainly rejected and its
    // remaining stations are skipped (the llk is then reported as -inf)
    const double floor_llk = (llk_floor && active && !resid) ? llk_floor[chain] : -INFINITY;
    bool stopped = false;
    int t_stop = ntiles;
    for (int t = 0; t < ntiles; ++t) {
        const int buf = t % STAGES;
        const uint32_t phase = (uint32_t)(t / STAGES) & 1u;
        const bool ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[buf], phase, kWaitLimit));
        if (!ok) {
            failed = true;
            break;
        }
        if (smask && !stopped) {
            // this tile's plan: the rectangles it integrates (node counts packed 5 + 5 bits per
            // rectangle) and the sides of the others
            const float4 tb = s_box[buf];
            const float bx0 = __fsub_rn(__fsub_rn(tb.x, x0h), x0l), bx1 = __fsub_rn(__fsub_rn(tb.y, x0h), x0l);
            const float by0 = __fsub_rn(__fsub_rn(tb.z, y0h), y0l), by1 = __fsub_rn(__fsub_rn(tb.w, y0h), y0l);
            uint32_t sides = smask & 0x0FFFu, qrect = 0u, qpack = 0u;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                int n1, n2;
                if ((smask >> (27 + r) & 1u) &&
                    tile_quad(C.rect[r], (smask >> (24 + r)) & 1u, bx0, bx1, by0, by1, n1, n2)) {
                    qrect |= 1u << r;
                    qpack |= (uint32_t)(n1 | (n2 << 5)) << (10 * r);
                    sides &= ~(0xFu << (4 * r));
                }
            }
            // one rectangle's nodes in this warp's buffer (every lane reads all of them); the
            // buffer is refilled only when it holds other nodes
            auto load_nodes = [&](int r) -> const float4* {
                const int n1 = (qpack >> (10 * r)) & 31, n2 = (qpack >> (10 * r + 5)) & 31;
                const int b = kNodeBufs == 3 ? r : 0;
                const uint64_t key = (uint64_t)(r | (n1 << 2) | (n2 << 7));
                if (((node_keys >> (12 * b)) & 0xFFFull) != key) {
                    __syncwarp();
                    if (lane < n1 * n2) s_node[warp][b][lane] = rect_node(C.rect[r], n1, n2, lane, s_gx, s_gw);
                    __syncwarp();
                    node_keys = (node_keys & ~(0xFFFull << (12 * b))) | (key << (12 * b));
                }
                return s_node[warp][b];
            };
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
                    resid[(size_t)chain * m_padded + (order ? __ldg(order + col) : col)] = (col < m) ? r : 0.f;
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
                    uint32_t msk = sides;
#pragma unroll 1
                    while (msk) {
                        const int sidx = __ffs(msk) - 1;
                        msk &= msk - 1;
                        side_pair<SV<SPL>>(ScalarSide(C.side[sidx]), Xr, Yr, ue, un, uv, (smask >> (kSides + sidx)) & 1u);
                    }
                    uint32_t qm = qrect;
#pragma unroll 1
                    while (qm) {
                        const int r = __ffs(qm) - 1;
                        qm &= qm - 1;
                        const float4* nodes = load_nodes(r);
                        rect_quad<SV<SPL>>(C.rect[r], nodes, ((qpack >> (10 * r)) & 31) * ((qpack >> (10 * r + 5)) & 31),
                                           Xr, Yr, ue, un, uv);
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
                    uint32_t msk = sides;
#pragma unroll 1
                    while (msk) {
                        const int sidx = __ffs(msk) - 1;
                        msk &= msk - 1;
                        side_pair<float>(ScalarSide(C.side[sidx]), Xr, Yr, ue, un, uv, (smask >> (kSides + sidx)) & 1u);
                    }
                    uint32_t qm = qrect;
#pragma unroll 1
                    while (qm) {
                        const int r = __ffs(qm) - 1;
                        qm &= qm - 1;
                        const float4* nodes = load_nodes(r);
                        rect_quad<float>(C.rect[r], nodes, ((qpack >> (10 * r)) & 31) * ((qpack >> (10 * r + 5)) & 31),
                                         Xr, Yr, ue, un, uv);
                    }
                    finish(ue, un, uv, j);
                }
            }
            if (floor_llk > -INFINITY && norm - 0.5 * warp_sum(ff_to_double(acc)) < floor_llk) stopped = true;
        }
        // done with this buffer: the last warp of the CTA to get here refills it
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            if (atomicAdd(&s_done[buf], 1) == WARPS - 1) {
                __threadfence_block();
                s_done[buf] = 0;
                if (t + STAGES < ntiles) {
                    fence_proxy_async_smem();
                    issue(t + STAGES, buf);
                    atomicAdd(&s_issued, 1);
                }
            }
        }
        // a CTA of one stopped warp leaves the ring; CTAs of several warps keep counting tiles
        // (the stopped warp's share of each tile's completion) without computing
        if (WARPS == 1 && stopped) {
            t_stop = t;
            break;
        }
    }
    if (WARPS == 1 && stopped && !failed) {
        // wait (bounded) for the copies already issued into this CTA's ring before it exits
        if (lane == 0) {
            const int last = s_issued;
            for (int t = t_stop + 1; t < last; ++t)
                mbar_wait_bounded(&full[t % STAGES], (uint32_t)(t / STAGES) & 1u, kWaitLimit);
        }
        __syncwarp();
        if (lane == 0) llk[chain] = -INFINITY;
        return;
    }
    if (__syncthreads_or(failed)) {
        // a wait gave up: drain the copies still in flight (bounded) before the CTA exits
        if (threadIdx.x == 0) {
            raise_flag(flags, DEV_ERR_TIMEOUT);
            const int last = s_issued;
            for (int t = (last > STAGES ? last - STAGES : 0); t < last; ++t)
                mbar_wait_bounded(&full[t % STAGES], (uint32_t)(t / STAGES) & 1u, kWaitLimit);
        }
        return;
    }
    const double sum = warp_sum(ff_to_double(acc));
    if (lane == 0 && active) llk[chain] = stopped ? -INFINITY : norm - 0.5 * sum;
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
                const int32_t* __restrict__ oid, const int32_t* __restrict__ order, int noffsets, int m,
                int m_padded, double norm, double* __restrict__ llk, float* __restrict__ resid,
                const int32_t* __restrict__ index, const int32_t* __restrict__ count) {
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
            if (resid && s_chain[c] < n)
                resid[(size_t)s_chain[c] * m_padded + (order ? __ldg(order + j) : j)] = (j < m) ? r : 0.f;
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
static constexpr CdmVariant kCdmVariants[] = {{8}, {4}, {4}, {2}, {4}, {4}, {2}, {4}, {4}, {4}, {4}, {1}, {1}, {1}, {2}};
static constexpr int kCdmVariantCount = 15;
// Mogi launch variants: chains per CTA held in registers (16, 8, 32)
static constexpr int kMogiChainsOf[] = {16, 8, 32};
static constexpr int kMogiVariantCount = 3;

extern "C" int32_t ag_forward_variants(int model) {
    return model == AG_MODEL_CDM ? kCdmVariantCount : model == AG_MODEL_MOGI ? kMogiVariantCount : 0;
}

// CDM workspace: compacted chain constants, the chain of each slot, the set-up header (slot
// count and cost histogram), each requested chain's cost bucket
static size_t al256(size_t b) { return (b + 255) / 256 * 256; }

extern "C" size_t ag_forward_workspace_bytes(int model, int32_t n) {
    if (model == AG_MODEL_CDM && n > 0)
        return al256((size_t)n * sizeof(ChainC)) + al256((size_t)n * sizeof(int32_t)) + al256(sizeof(SetupHdr)) +
               al256((size_t)n);
    return 0;
}

static int check_stations(const ag_station_set* st) {
    AG_REQUIRE(st != nullptr, "stations is NULL");
    AG_REQUIRE(st->xy && st->losd && st->weight, "station arrays must not be NULL");
    AG_REQUIRE(st->m > 0 && st->m_padded >= st->m && st->m_padded % AG_STATION_TILE == 0,
               "m=%d m_padded=%d: m_padded must be a multiple of %d and >= m", st->m,
               st->m_padded, AG_STATION_TILE);
    AG_REQUIRE(aligned(st->xy, 16) && aligned(st->losd, 16) && aligned(st->weight, 16) &&
                   (st->oid == nullptr || aligned(st->oid, 16)) && (st->order == nullptr || aligned(st->order, 4)),
               "station arrays must be 16-byte aligned (order 4-byte)");
    return AG_OK;
}

static int forward_llk(int model, const ag_layout* layout, const double* theta, int32_t n,
                       const ag_station_set* st, double norm, const uint32_t* mask_in,
                       const int32_t* index, const int32_t* count, const double* llk_floor, double* llk,
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
        AG_REQUIRE(st->tile_box != nullptr && aligned(st->tile_box, 16),
                   "the CDM needs the stations' tile boxes (ag_station_boxes), 16-byte aligned");
        const float4* tile_box = reinterpret_cast<const float4*>(st->tile_box);
        const int ntiles = st->m_padded / AG_STATION_TILE;
        ChainC* chains = reinterpret_cast<ChainC*>(workspace);
        int32_t* slot_chain = reinterpret_cast<int32_t*>(static_cast<char*>(workspace) +
                                                         al256((size_t)n * sizeof(ChainC)));
        SetupHdr* hdr = reinterpret_cast<SetupHdr*>(reinterpret_cast<char*>(slot_chain) +
                                                    al256((size_t)n * sizeof(int32_t)));
        int8_t* key = reinterpret_cast<int8_t*>(reinterpret_cast<char*>(hdr) + al256(sizeof(SetupHdr)));
        int32_t* nslots = &hdr->nslots;
        rc = cuda_status(cudaMemsetAsync(hdr, 0, sizeof(SetupHdr), s), "cudaMemsetAsync(set-up header)");
        if (rc) return rc;
        cdm_cost_kernel<<<(n + 127) / 128, 128, 0, s>>>(L, theta, n, mask_in, chain_status, index, count, tile_box,
                                                        ntiles, key, hdr);
        rc = launch_status("cdm_cost_kernel");
        if (rc) return rc;
        cdm_setup_kernel<<<(n + 127) / 128, 128, 0, s>>>(L, theta, n, key, chains, noffsets, index, count,
                                                         slot_chain, hdr);
        rc = launch_status("cdm_setup_kernel");
        if (rc) return rc;
        const int v = L.variant;
        AG_REQUIRE(v >= 0 && v < kCdmVariantCount, "CDM variant %d out of range [0, %d)", v, kCdmVariantCount);
        const int warps = kCdmVariants[v].warps;
        const int grid = (n + warps - 1) / warps;
#define AG_CDM_LAUNCH(W, B, SPL, ST)                                                                    \
    cdm_llk_kernel<W, B, SPL, ST><<<grid, W * 32, 0, s>>>(chains, slot_chain, nslots, n, xy, ld, st->weight, \
                                                          st->oid, tile_box, st->order, st->m, st->m_padded,     \
                                                          norm, llk_floor, llk, residuals, nullptr)
        // warps per CTA, CTAs per SM, stations per lane, ring depth; a CTA of one warp has its
        // own ring, so its chain never waits for another chain's tiles
        switch (v) {
            case 0: AG_CDM_LAUNCH(8, 2, 1, 4); break;
            case 1: AG_CDM_LAUNCH(4, 4, 1, 4); break;
            case 2: AG_CDM_LAUNCH(4, 5, 1, 4); break;
            case 3: AG_CDM_LAUNCH(2, 8, 1, 4); break;
            case 4: AG_CDM_LAUNCH(4, 3, 2, 4); break;
            case 5: AG_CDM_LAUNCH(4, 4, 2, 4); break;
            case 6: AG_CDM_LAUNCH(2, 6, 2, 4); break;
            case 7: AG_CDM_LAUNCH(4, 2, 4, 4); break;
            case 8: AG_CDM_LAUNCH(4, 3, 4, 4); break;
            case 9: AG_CDM_LAUNCH(4, 4, 4, 4); break;
            case 10: AG_CDM_LAUNCH(4, 5, 4, 4); break;
            case 11: AG_CDM_LAUNCH(1, 12, 4, 2); break;
            case 12: AG_CDM_LAUNCH(1, 12, 4, 3); break;
            case 13: AG_CDM_LAUNCH(1, 10, 4, 3); break;
            default: AG_CDM_LAUNCH(2, 6, 4, 3); break;
        }
#undef AG_CDM_LAUNCH
        return launch_status("cdm_llk_kernel");
    }
    if (model == AG_MODEL_MOGI) {
        AG_REQUIRE(L.nsources == 1 || L.nsources == 2, "1 or 2 Mogi sources are supported");
        AG_REQUIRE(L.variant >= 0 && L.variant < kMogiVariantCount, "Mogi variant %d out of range [0, %d)",
                   L.variant, kMogiVariantCount);
        const int ch = kMogiChainsOf[L.variant];
        const int grid = (n + ch - 1) / ch;
#define AG_MOGI_LAUNCH(CH, NS)                                                                               \
    mogi_llk_kernel<CH, NS><<<grid, 256, 0, s>>>(L, theta, n, mask_in, xy, ld, st->weight, st->oid, st->order, \
                                                 noffsets, st->m, st->m_padded, norm, llk, residuals, index, count)
        if (L.nsources == 1) {
            if (ch == 8) AG_MOGI_LAUNCH(8, 1);
            else if (ch == 32) AG_MOGI_LAUNCH(32, 1);
            else AG_MOGI_LAUNCH(16, 1);
        } else {
            if (ch == 8) AG_MOGI_LAUNCH(8, 2);
            else if (ch == 32) AG_MOGI_LAUNCH(32, 2);
            else AG_MOGI_LAUNCH(16, 2);
        }
#undef AG_MOGI_LAUNCH
        return launch_status("mogi_llk_kernel");
    }
    return set_error(AG_ERR_ARG, "unknown model %d", model);
}

extern "C" int ag_forward_llk(int model, const ag_layout* layout, const double* theta, int32_t n,
                              const ag_station_set* st, double norm, const uint32_t* mask_in,
                              double* llk, uint32_t* chain_status, float* residuals,
                              void* workspace, size_t workspace_bytes, void* stream) {
    return forward_llk(model, layout, theta, n, st, norm, mask_in, nullptr, nullptr, nullptr, llk, chain_status,
                       residuals, workspace, workspace_bytes, stream);
}

extern "C" int ag_forward_llk_floor(int model, const ag_layout* layout, const double* theta, int32_t n,
                                    const ag_station_set* st, double norm, const uint32_t* mask_in,
                                    const double* llk_floor, double* llk, uint32_t* chain_status,
                                    void* workspace, size_t workspace_bytes, void* stream) {
    AG_REQUIRE(llk_floor != nullptr, "llk_floor must not be NULL (ag_forward_llk evaluates without one)");
    return forward_llk(model, layout, theta, n, st, norm, mask_in, nullptr, nullptr, llk_floor, llk, chain_status,
                       nullptr, workspace, workspace_bytes, stream);
}

extern "C" int ag_forward_llk_subset_floor(int model, const ag_layout* layout, const double* theta, int32_t n,
                                           const ag_station_set* st, double norm, const int32_t* index,
                                           const int32_t* count, const double* llk_floor, double* llk,
                                           uint32_t* chain_status, void* workspace, size_t workspace_bytes,
                                           void* stream) {
    AG_REQUIRE(index != nullptr && count != nullptr && llk_floor != nullptr,
               "index, count and llk_floor must not be NULL");
    return forward_llk(model, layout, theta, n, st, norm, nullptr, index, count, llk_floor, llk, chain_status,
                       nullptr, workspace, workspace_bytes, stream);
}

extern "C" int ag_forward_llk_subset(int model, const ag_layout* layout, const double* theta,
                                     int32_t n, const ag_station_set* st, double norm,
                                     const int32_t* index, const int32_t* count, double* llk,
                                     uint32_t* chain_status, float* residuals, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    AG_REQUIRE(index != nullptr && count != nullptr, "index and count must not be NULL");
    return forward_llk(model, layout, theta, n, st, norm, nullptr, index, count, nullptr, llk, chain_status,
                       residuals, workspace, workspace_bytes, stream);
}

extern "C" int ag_cdm_work(const ag_layout* layout, const double* theta, int32_t n, const ag_station_set* st,
                           double* flop, double* sfu, void* stream) {
    AG_REQUIRE(layout && theta && flop && n > 0, "invalid arguments");
    int rc = check_stations(st);
    if (rc) return rc;
    AG_REQUIRE(st->tile_box != nullptr && aligned(st->tile_box, 16),
               "the CDM needs the stations' tile boxes (ag_station_boxes), 16-byte aligned");
    const ag_layout L = *layout;
    AG_REQUIRE(L.nparams > 0 && L.axes_idx >= 0 && L.axes_idx + 2 < L.nparams && L.omega_idx >= 0 &&
                   L.omega_idx + 2 < L.nparams,
               "invalid CDM layout");
    cdm_work_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(
        L, theta, n, reinterpret_cast<const float4*>(st->tile_box), st->m, flop, sfu);
    return launch_status("cdm_work_kernel");
}

extern "C" int ag_station_boxes(const float* xy, int32_t m, int32_t m_padded, float* tile_box, void* stream) {
    AG_REQUIRE(xy && tile_box && m > 0 && m_padded >= m && m_padded % AG_STATION_TILE == 0,
               "invalid arguments (m=%d, m_padded=%d must be a multiple of %d)", m, m_padded, AG_STATION_TILE);
    AG_REQUIRE(aligned(xy, 16) && aligned(tile_box, 16), "xy and tile_box must be 16-byte aligned");
    const int ntiles = m_padded / AG_STATION_TILE;
    station_boxes_kernel<<<(ntiles + 7) / 8, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const float4*>(xy), m, ntiles, reinterpret_cast<float4*>(tile_box));
    return launch_status("station_boxes_kernel");
}

extern "C" int ag_cdm_check(const ag_layout* layout, const double* theta, int32_t n,
                            uint32_t* chain_status, void* stream) {
    AG_REQUIRE(layout && theta && chain_status && n > 0, "invalid arguments");
    cdm_check_kernel<<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(*layout, theta, n, chain_status);
    return launch_status("cdm_check_kernel");
}
