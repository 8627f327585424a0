// Per-stage CATMIP kernels: prior, Metropolis proposal/accept, COV β schedule,
// weighted covariance, Cholesky, multinomial resampling, scaling adaptation.
//
// Every kernel is a fixed launch shape on the caller's stream with all
// data-dependent control flow kept on the device (a "done" flag in the
// schedule state instead of host round trips), so one annealing stage can be
// captured into one CUDA graph.  All reductions run in a fixed order, so
// repeated runs are bitwise identical.
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace ag {

constexpr int kMaxP = 32;          // parameter counts up to this use the one-thread-per-chain proposal
constexpr int kMaxPLarge = 512;    // largest parameter count of the stage kernels
constexpr int kGridPoints = 11;    // COV.cc:276 Nbeta = 10 -> 11 points per level
constexpr int kBrentMaxIter = 128;   // Brent iterations run on the device per stage
constexpr int kGridLevels = 11;    // COV.cc:313 Nloop <= Nbeta
constexpr int kEvalChunk = 1024;   // chains per CTA in a COV evaluation
constexpr int kSigmaChunk = 256;   // chains per CTA in the covariance

// ---------------------------------------------------------------------------
// prior
__global__ void prior_sample_kernel(int n, int p, const double* __restrict__ lo,
                                    const double* __restrict__ hi, uint64_t seed, uint32_t attempt,
                                    const uint32_t* __restrict__ redraw, double* __restrict__ theta) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (redraw && !redraw[i]) return;
    for (int j = 0; j < p; ++j) {
        u32x4 r = draw(seed, (uint32_t)i, (uint32_t)j, STREAM_PRIOR, 0u, attempt);
        double u = u01_closed_open(r.x, r.y);
        // gsl_ran_flat: a (1 - u) + b u
        theta[(size_t)i * p + j] = lo[j] * (1.0 - u) + hi[j] * u;
    }
}

__device__ inline double uniform_log_prior(int p, const double* lo, const double* hi) {
    double s = 0.0;
    for (int j = 0; j < p; ++j) s -= log(hi[j] - lo[j]);
    return s;
}

__global__ void prior_llk_kernel(const double* __restrict__ theta, int n, int p,
                                 const double* __restrict__ lo, const double* __restrict__ hi,
                                 uint32_t* __restrict__ mask, double* __restrict__ prior) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    bool out = false;
    for (int j = 0; j < p; ++j) {
        double v = theta[(size_t)i * p + j];
        out |= !(lo[j] <= v && v <= hi[j]);
    }
    if (mask && out) mask[i] |= CHAIN_OUT_OF_SUPPORT;
    if (prior) prior[i] = uniform_log_prior(p, lo, hi);
}

// ---------------------------------------------------------------------------
// Metropolis proposal, verify and prior (Metropolis.py:160-183, 236-259)
__global__ void propose_kernel(const double* __restrict__ theta, int n, int p,
                               const double* __restrict__ chol, const double* __restrict__ lo,
                               const double* __restrict__ hi, uint64_t seed, uint32_t step,
                               const uint32_t* __restrict__ epoch, double* __restrict__ cand,
                               uint32_t* __restrict__ mask, double* __restrict__ cprior, int chain0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t ep = *epoch;
    double z[kMaxP];
    for (int j = 0; j < p; j += 2) {
        double z0, z1;
        normal_pair(draw(seed, (uint32_t)(chain0 + i), (uint32_t)(j >> 1), STREAM_PROPOSAL, step, ep), z0, z1);
        z[j] = z0;
        if (j + 1 < p) z[j + 1] = z1;
    }
    const double* th = theta + (size_t)i * p;
    double* c = cand + (size_t)i * p;
    bool out = false;
    for (int j = 0; j < p; ++j) {
        double d = 0.0;
        for (int k = 0; k <= j; ++k) d = fma(chol[j * p + k], z[k], d);
        double v = th[j] + d;
        c[j] = v;
        out |= !(lo[j] <= v && v <= hi[j]);
    }
    if (out)
        for (int j = 0; j < p; ++j) c[j] = th[j];
    mask[i] = out ? CHAIN_OUT_OF_SUPPORT : 0u;
    cprior[i] = uniform_log_prior(p, lo, hi);
}

// The same proposal for many parameters: one warp per chain, the chain's normals in
// shared memory, lane j computing the rows j, j + 32, ... of L z with the same
// sequential k order as propose_kernel (identical results).
constexpr int kProposeWarps = 8;
__global__ void __launch_bounds__(kProposeWarps * 32)
propose_warp_kernel(const double* __restrict__ theta, int n, int p, const double* __restrict__ chol,
                    const double* __restrict__ lo, const double* __restrict__ hi, uint64_t seed,
                    uint32_t step, const uint32_t* __restrict__ epoch, double* __restrict__ cand,
                    uint32_t* __restrict__ mask, double* __restrict__ cprior, int chain0) {
    extern __shared__ double sz[];                 // [kProposeWarps][p] normals
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = blockIdx.x * kProposeWarps + warp;
    if (i >= n) return;
    double* z = sz + (size_t)warp * p;
    const uint32_t ep = *epoch;
    for (int q = lane; 2 * q < p; q += 32) {
        double z0, z1;
        normal_pair(draw(seed, (uint32_t)(chain0 + i), (uint32_t)q, STREAM_PROPOSAL, step, ep), z0, z1);
        z[2 * q] = z0;
        if (2 * q + 1 < p) z[2 * q + 1] = z1;
    }
    __syncwarp();
    const double* th = theta + (size_t)i * p;
    double* c = cand + (size_t)i * p;
    bool out = false;
    for (int j = lane; j < p; j += 32) {
        const double* row = chol + (size_t)j * p;
        double d = 0.0;
        for (int k = 0; k <= j; ++k) d = fma(row[k], z[k], d);
        const double v = th[j] + d;
        c[j] = v;
        out |= !(lo[j] <= v && v <= hi[j]);
    }
    out = __any_sync(0xffffffffu, out);
    if (out)
        for (int j = lane; j < p; j += 32) c[j] = th[j];
    if (lane == 0) {
        mask[i] = out ? CHAIN_OUT_OF_SUPPORT : 0u;
        cprior[i] = uniform_log_prior(p, lo, hi);
    }
}

// ---------------------------------------------------------------------------
// Metropolis accept/reject (Metropolis.py:185-223)
__global__ void accept_kernel(int n, int p, const double* __restrict__ beta, uint64_t seed,
                              uint32_t step, const uint32_t* __restrict__ epoch,
                              const uint32_t* __restrict__ mask, const double* __restrict__ cand,
                              const double* __restrict__ cprior, const double* __restrict__ cdata,
                              double* __restrict__ theta, double* __restrict__ prior,
                              double* __restrict__ data, double* __restrict__ post,
                              unsigned long long* __restrict__ counters, int chain0) {
    __shared__ unsigned int s_cnt[3];
    if (threadIdx.x < 3) s_cnt[threadIdx.x] = 0u;
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if (mask[i]) {
            atomicAdd(&s_cnt[1], 1u);
        } else {
            const double b = *beta;
            const double cp = cprior[i] + b * cdata[i];
            u32x4 r = draw(seed, (uint32_t)(chain0 + i), 0u, STREAM_ACCEPT, step, *epoch);
            const double u = u01_open_closed(r.x, r.y);
            if (log(u) > cp - post[i]) {
                atomicAdd(&s_cnt[2], 1u);
            } else {
                atomicAdd(&s_cnt[0], 1u);
                for (int j = 0; j < p; ++j) theta[(size_t)i * p + j] = cand[(size_t)i * p + j];
                prior[i] = cprior[i];
                data[i] = cdata[i];
                post[i] = cp;
            }
        }
    }
    __syncthreads();
    if (threadIdx.x < 3 && s_cnt[threadIdx.x])
        atomicAdd(&counters[threadIdx.x], (unsigned long long)s_cnt[threadIdx.x]);
}

// The data log-likelihood below which each proposal is certainly rejected (early rejection,
// Solonen et al. 2012, Bayesian Analysis 7(3)).  accept_kernel rejects when
// log u > cprior + β cdata − post; with the same uniform u, every cdata below
// (post + log u − cprior)/β is rejected.  The floor is lowered by a relative 1e-9 so that a
// likelihood evaluation stopped below it is rejected whatever the rounding of the test;
// chains outside the support, and β = 0, get -inf (never stopped).
__global__ void accept_floor_kernel(int n, const double* __restrict__ beta, uint64_t seed, uint32_t step,
                                    const uint32_t* __restrict__ epoch, const uint32_t* __restrict__ mask,
                                    const double* __restrict__ cprior, const double* __restrict__ post,
                                    double* __restrict__ floor, int chain0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double b = *beta;
    double f = -INFINITY;
    if (!mask[i] && b > 0.0) {
        u32x4 r = draw(seed, (uint32_t)(chain0 + i), 0u, STREAM_ACCEPT, step, *epoch);
        const double u = u01_open_closed(r.x, r.y);
        f = (post[i] + log(u) - cprior[i]) / b;
        f -= (fabs(f) + 1.0) * 1e-9;
        if (!(f == f)) f = -INFINITY;
    }
    floor[i] = f;
}

__global__ void posterior_kernel(int n, const double* __restrict__ beta,
                                 const double* __restrict__ prior, const double* __restrict__ data,
                                 double* __restrict__ post) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) post[i] = prior[i] + (*beta) * data[i];
}

// ---------------------------------------------------------------------------
// COV β schedule (COV.cc:222-368).
struct CovState {
    double median;
    double llk_max;
    double beta0;          // β at the start of the stage
    double low, high, step;
    double pts[kGridPoints];
    double cov_high;       // COV at the full remaining δβ
    double dbeta;          // chosen δβ
    double cov;            // COV at dbeta
    double s1;             // shifted weight sum at dbeta
    int npts;              // points to evaluate in the next round
    int level;             // levels done (Nloop)
    int done;
    int skip;              // jumped straight to β = 1
    // Brent's method (minimisation of (COV - target)² on [low, high])
    double a, b, x, w, v, fx, fw, fv, d, e, u;
    int iter;
    int phase;             // 0: evaluating the initial point, 1: iterating
};

// order-preserving map of a double onto uint64
__device__ inline uint64_t dkey(double x) {
    uint64_t b = (uint64_t)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ inline double dkey_inv(uint64_t k) {
    uint64_t b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    return __longlong_as_double((long long)b);
}

// k-th smallest (0-based) key of llk by 8-bit radix select; one CTA
__device__ uint64_t block_select(const double* __restrict__ llk, int n, int k, int* hist,
                                 int* sh) {
    uint64_t prefix = 0ull, mask = 0ull;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 56 - 8 * pass;
        for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            uint64_t key = dkey(llk[i]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 255], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0, d = 0;
            for (; d < 256; ++d) {
                if (acc + hist[d] > k) break;
                acc += hist[d];
            }
            sh[0] = d;
            sh[1] = k - acc;
        }
        __syncthreads();
        const int d = sh[0];
        k = sh[1];
        prefix |= (uint64_t)d << shift;
        mask |= 255ull << shift;
        __syncthreads();
    }
    return prefix;
}

__global__ void __launch_bounds__(1024) cov_median_kernel(const double* __restrict__ llk, int n,
                                                          const double* __restrict__ beta,
                                                          CovState* __restrict__ S) {
    __shared__ int hist[256];
    __shared__ int sh[2];
    __shared__ double smax[32];
    // maximum
    double mx = -INFINITY;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, llk[i]);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
    __syncthreads();
    // median as gsl_stats_median_from_sorted_data: mean of elements (n-1)/2 and n/2
    const uint64_t klo = block_select(llk, n, (n - 1) / 2, hist, sh);
    const uint64_t khi = (n % 2) ? klo : block_select(llk, n, n / 2, hist, sh);
    if (threadIdx.x == 0) {
        double m = smax[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, smax[w]);
        const double lo = dkey_inv(klo), hi = dkey_inv(khi);
        S->median = (n % 2) ? lo : (lo + hi) / 2.0;
        S->llk_max = m;
        S->beta0 = *beta;
        S->low = 0.0;
        S->high = 1.0 - *beta;
        S->step = 0.0;
        S->pts[0] = S->high;     // round 0 evaluates the full remaining step
        S->npts = 1;
        S->level = 0;
        S->done = 0;
        S->skip = 0;
    }
}

// shifted weight moments Σe and Σe², e = exp(g (llk − median) − g (llk_max − median)), of one
// chunk of kEvalChunk chains: 256 threads each sum their chains in index order, then the warps'
// sums are added in warp order
__device__ void chunk_moments(const double* __restrict__ llk, int n, double g, double med, double llk_max,
                              int chunk, double* __restrict__ out) {
    __shared__ double r1[8], r2[8];
    const double mx = g * (llk_max - med);
    double s1 = 0.0, s2 = 0.0;
    const int begin = chunk * kEvalChunk;
    const int end = min(n, begin + kEvalChunk);
    for (int i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const double e = exp(g * (llk[i] - med) - mx);
        s1 += e;
        s2 = fma(e, e, s2);
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if ((threadIdx.x & 31) == 0) {
        r1[threadIdx.x >> 5] = s1;
        r2[threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a += r1[w];
            b += r2[w];
        }
        out[0] = a;
        out[1] = b;
    }
    __syncthreads();      // r1 and r2 are reused by the next chunk
}

// COV of the normalised weights from the shifted moments, with the reference's
// convention that a non-finite COV counts as 1e100 (COV.cc:355-364)
__device__ double cov_from_moments(double s1, double s2, double mx, int n) {
    // an infinite weight in the reference (exp overflow) or an infinite weight sum
    if (isinf(exp(mx)) || !(s1 > 0.0) || isinf(exp(mx) * s1)) return 1e100;
    double v = (s2 / (s1 * s1) - 1.0 / n) / (double)(n - 1);
    if (v < 0.0) v = 0.0;
    double c = (double)n * sqrt(v);
    if (!isfinite(c)) return 1e100;
    return c;
}

// One level of the grid search (COV.cc:240-326) given the COVs of this round's points: round 0
// evaluated the full remaining step, later rounds the kGridPoints points of a level.
__device__ void grid_step(CovState& S, const double* cov, double target, double tol) {
    const double Nbeta = 10.0;
    if (S.level == 0) {
        // skip straight to β = 1 (COV.cc:257-268)
        S.cov_high = cov[0];
        if (cov[0] < target || fabs(cov[0] - target) < tol) {
            S.done = 1;
            S.skip = 1;
            S.dbeta = S.high;
            return;
        }
    } else {
        // scan of one level (COV.cc:287-311)
        bool found = false;
        int nb = 0;
        for (; nb < S.npts; ++nb) {
            if (fabs(cov[nb] - target) < tol) { found = true; break; }
            if (cov[nb] >= target) { if (nb == 0) found = true; break; }
        }
        const double step = S.step;
        // a completed scan leaves the reference's accumulator one step past the last
        // point and steps it back (COV.cc:301), which can differ from that point in the
        // last bit
        const double guess = (nb < S.npts) ? S.pts[nb] : (S.pts[S.npts - 1] + step) - step;
        S.high = guess;
        S.low = guess - step;
        if (found || S.level >= kGridLevels) {
            S.done = 1;
            S.dbeta = guess;
            return;
        }
    }
    // next level: points low, low + step, ... accumulated as the reference does
    S.level += 1;
    const double step = (S.high - S.low) / Nbeta;
    S.step = step;
    double g = S.low;
    for (int k = 0; k < kGridPoints; ++k) {
        S.pts[k] = g;
        g += step;
    }
    S.npts = kGridPoints;
}

// Brent's minimiser for δβ (COV.cc:58-219).  The reference minimises f(δβ) = (COV − target)²
// with GSL's Brent minimiser, primed with the guess δβ = 5e-5 inside [0, 1 − β], and stops
// when the COV at the latest evaluated point is within tol of the target (or after maxiter
// iterations), returning the best point found.  GSL is not part of the reference, so the
// iteration itself is Brent's published method (R. P. Brent, "Algorithms for Minimization
// without Derivatives", 1973, ch. 5, procedure localmin: parabolic interpolation through the
// three best points, golden-section steps when the parabola is unacceptable) restated here.
// One call per evaluation round: the COVs of the points of the previous round come in as
// cov[], the next point goes out through S.pts.
__device__ inline double brent_metric(double cov, double target) {
    return (cov >= 1e100) ? 1e100 : (cov - target) * (cov - target);
}

__device__ void brent_step(CovState& S, const double* cov, double target, double tol, int maxiter) {
    const double golden = 0.3819660112501051;      // (3 − √5) / 2
    if (S.level == 0) {
        // full remaining step first: skip straight to β = 1 if it meets the target (COV.cc:103-116)
        S.cov_high = cov[0];
        if (cov[0] < target || fabs(cov[0] - target) < tol) {
            S.done = 1;
            S.skip = 1;
            S.dbeta = S.high;
            return;
        }
        // bracket [0, 1 − β], first point the reference's guess, interior point v = w at the
        // golden section of the bracket; both evaluated in the next round
        S.level = 1;
        S.a = 0.0;
        S.b = S.high;
        S.x = (5.0e-5 < S.high) ? 5.0e-5 : 0.5 * S.high;
        S.v = S.w = S.a + golden * (S.b - S.a);
        S.d = S.e = 0.0;
        S.iter = 0;
        S.phase = 0;
        S.pts[0] = S.x;
        S.pts[1] = S.v;
        S.npts = 2;
        return;
    }
    if (S.phase == 0) {
        S.fx = brent_metric(cov[0], target);
        S.fv = S.fw = brent_metric(cov[1], target);
        S.phase = 1;
    } else {
        // fold the new point u into the bracket and the three best points
        const double u = S.u, fu = brent_metric(cov[0], target);
        if (fu <= S.fx) {
            if (u < S.x) S.b = S.x; else S.a = S.x;
            S.v = S.w; S.fv = S.fw;
            S.w = S.x; S.fw = S.fx;
            S.x = u; S.fx = fu;
        } else {
            if (u < S.x) S.a = u; else S.b = u;
            if (fu <= S.fw || S.w == S.x) {
                S.v = S.w; S.fv = S.fw;
                S.w = u; S.fw = fu;
            } else if (fu <= S.fv || S.v == S.x || S.v == S.w) {
                S.v = u; S.fv = fu;
            }
        }
        S.iter += 1;
        // the reference's convergence test is on the COV of the latest point (COV.cc:182)
        if (fabs(cov[0] - target) < tol || S.iter >= maxiter) {
            S.done = 1;
            S.dbeta = S.x;
            return;
        }
    }
    // next point
    const double x = S.x, a = S.a, b = S.b;
    const double xm = 0.5 * (a + b);
    const double tol1 = 1.4901161193847656e-08 * fabs(x) + 1e-15;   // √ε·|x| plus an absolute floor
    const double tol2 = 2.0 * tol1;
    if (fabs(x - xm) <= tol2 - 0.5 * (b - a)) {                     // bracket down to the tolerance
        S.done = 1;
        S.dbeta = x;
        return;
    }
    double d = S.d, e = S.e;
    bool parabolic = false;
    if (fabs(e) > tol1) {
        double r = (x - S.w) * (S.fx - S.fv);
        double q = (x - S.v) * (S.fx - S.fw);
        double pp = (x - S.v) * q - (x - S.w) * r;
        q = 2.0 * (q - r);
        if (q > 0.0) pp = -pp; else q = -q;
        const double e_prev = e;
        e = d;
        if (fabs(pp) < fabs(0.5 * q * e_prev) && pp > q * (a - x) && pp < q * (b - x)) {
            d = pp / q;
            const double u = x + d;
            if (u - a < tol2 || b - u < tol2) d = (xm >= x) ? tol1 : -tol1;
            parabolic = true;
        }
    }
    if (!parabolic) {
        e = (x >= xm) ? a - x : b - x;
        d = golden * e;
    }
    const double u = (fabs(d) >= tol1) ? x + d : x + ((d >= 0.0) ? tol1 : -tol1);
    S.d = d;
    S.e = e;
    S.u = u;
    S.pts[0] = u;
    S.npts = 1;
}

// Grid-wide barrier of a cooperative launch (every block of the grid is resident).  The
// barrier words (arrival count, generation) are cleared by the host before the launch and
// the count returns to zero at every barrier.  A block that waits more than kBarrierLimit
// polls raises DEV_ERR_TIMEOUT and returns false; every later barrier then gives up too, so a
// lost block ends the kernel with the flag set instead of hanging it.
constexpr uint32_t kBarrierLimit = 1u << 22;
struct __align__(256) GridBarrier {
    unsigned count;
    unsigned gen;
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ bool grid_sync(GridBarrier* bar, uint32_t* flags) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_gpu(&bar->gen);
        __threadfence();
        int ok = 1;
        if (atomicAdd(&bar->count, 1u) == gridDim.x - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            uint32_t polls = 0;
            while (ld_acquire_gpu(&bar->gen) == gen) {
                if (++polls > kBarrierLimit) {
                    ok = 0;
                    raise_flag(flags, DEV_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// The whole δβ search of one stage and its weights in one cooperative launch (COV.cc:58-368).
// Each round, the blocks evaluate the (point, chunk) moments of the round's points, meet at a
// grid barrier, and then every block adds the partials in chunk order and takes the same
// decision on its own copy of the search state, so a round needs one barrier.  The partials
// alternate between two buffers, so a block that starts the next round cannot overwrite
// partials that a slower block is still adding.  Then the moments at the chosen δβ, one more
// barrier, and the normalised weights.  Sums and decisions are those of one chunk per CTA and
// a sequential total over the chunks, whatever the grid size.
template <bool BRENT>
__global__ void __launch_bounds__(256) cov_schedule_kernel(const double* __restrict__ llk, int n, double target,
                                                           double tol, int maxiter, int rounds,
                                                           CovState* __restrict__ S, double* __restrict__ part,
                                                           GridBarrier* __restrict__ bar, double* __restrict__ beta,
                                                           double* __restrict__ dbeta_cov, double* __restrict__ w,
                                                           uint32_t* __restrict__ flags) {
    __shared__ CovState sS;
    __shared__ double s_tot[2 * kGridPoints];
    if (threadIdx.x == 0) sS = *S;        // median, maximum and the first round's point
    __syncthreads();
    const int nblk = (n + kEvalChunk - 1) / kEvalChunk;
    const size_t pbuf = (size_t)kGridPoints * nblk * 2;
    const double med = sS.median, lmax = sS.llk_max;
    for (int round = 0; round < rounds && !sS.done; ++round) {
        double* pr = part + (size_t)(round & 1) * pbuf;
        const int npts = sS.npts;
        for (int it = blockIdx.x; it < npts * nblk; it += gridDim.x) {
            const int pt = it / nblk, c = it - pt * nblk;
            chunk_moments(llk, n, sS.pts[pt], med, lmax, c, pr + ((size_t)pt * nblk + c) * 2);
        }
        if (!grid_sync(bar, flags)) return;
        if ((int)threadIdx.x < 2 * npts) {
            const int pt = threadIdx.x >> 1, m = threadIdx.x & 1;
            double a = 0.0;
            for (int k = 0; k < nblk; ++k) a += __ldcg(pr + ((size_t)pt * nblk + k) * 2 + m);
            s_tot[threadIdx.x] = a;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double cov[kGridPoints];
            for (int pt = 0; pt < npts; ++pt)
                cov[pt] = cov_from_moments(s_tot[2 * pt], s_tot[2 * pt + 1], sS.pts[pt] * (lmax - med), n);
            if (BRENT)
                brent_step(sS, cov, target, tol, maxiter);
            else
                grid_step(sS, cov, target, tol);
        }
        __syncthreads();
    }
    // moments at the chosen δβ, then the state, β, and the normalised weights
    double* fp = part + 2 * pbuf;
    const double g = sS.dbeta;
    for (int c = blockIdx.x; c < nblk; c += gridDim.x) chunk_moments(llk, n, g, med, lmax, c, fp + 2 * c);
    if (!grid_sync(bar, flags)) return;
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < nblk; ++k) {
            a += __ldcg(fp + 2 * k);
            b += __ldcg(fp + 2 * k + 1);
        }
        sS.s1 = a;
        sS.cov = cov_from_moments(a, b, g * (lmax - med), n);
        if (blockIdx.x == 0) {
            *S = sS;
            // β bookkeeping (COV.cc:264, 323)
            *beta = sS.skip ? 1.0 : sS.beta0 + sS.dbeta;
            dbeta_cov[0] = sS.dbeta;
            dbeta_cov[1] = sS.cov;
        }
    }
    __syncthreads();
    const double s1 = sS.s1, mx = g * (lmax - med);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = exp(g * (llk[i] - med) - mx) / s1;
}

// ---------------------------------------------------------------------------
// weighted covariance (COV.py:106-156): per-chunk partial sums in fixed order.  A chunk
// holds as many chains as fit the shared-memory budget (256 for up to 32 parameters).
constexpr size_t kSigmaSmem = 96 * 1024;
static int sigma_chunk(int p) {
    int c = kSigmaChunk;
    while (c > 1 && (size_t)c * (p + 1) * sizeof(double) > kSigmaSmem) c >>= 1;
    return c;
}

constexpr int kSigmaBlocks = 256;  // at most this many partial sums per entry

// Block b sums the chunks [b·cpb, (b+1)·cpb) in order into part[b][e]; the last block to
// finish adds the blocks' partials in block order and assembles Σ.
__global__ void __launch_bounds__(256) sigma_kernel(const double* __restrict__ theta,
                                                    const double* __restrict__ w, int n, int p, int chunk,
                                                    int cpb, double* __restrict__ part, double* __restrict__ tot,
                                                    unsigned* __restrict__ done, double* __restrict__ sigma) {
    extern __shared__ double sm[];      // [chunk][p] θ, then [chunk] w
    double* sth = sm;
    double* sw = sm + (size_t)chunk * p;
    // entries: 0 = Σw, 1..p = Σ w θ_a, then lower triangle (a >= b) Σ w θ_a θ_b
    const int nent = 1 + p + p * (p + 1) / 2;
    const int c0 = blockIdx.x * cpb;
    for (int c = c0; c < c0 + cpb; ++c) {
        const int begin = c * chunk;
        if (begin >= n) break;
        const int cnt = min(chunk, n - begin);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt * p; k += blockDim.x) sth[k] = theta[(size_t)begin * p + k];
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) sw[k] = w[begin + k];
        __syncthreads();
        for (int e = threadIdx.x; e < nent; e += blockDim.x) {
            int a = -1, b = -1;
            if (e >= 1 && e <= p) {
                a = e - 1;
            } else if (e > p) {
                // row a of the lower triangle starts at entry a (a + 1) / 2
                int t = e - 1 - p;
                a = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
                while ((a + 1) * (a + 2) / 2 <= t) ++a;
                while (a * (a + 1) / 2 > t) --a;
                b = t - a * (a + 1) / 2;
            }
            double acc = (c == c0) ? 0.0 : part[(size_t)blockIdx.x * nent + e];
            for (int i = 0; i < cnt; ++i) {
                double v = sw[i];
                if (a >= 0) v *= sth[i * p + a];
                if (b >= 0) v *= sth[i * p + b];
                acc += v;
            }
            part[(size_t)blockIdx.x * nent + e] = acc;
        }
    }
    // the last block to finish (threadfence reduction: the count is cleared before the launch)
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // totals over the blocks, in block order
    for (int e = threadIdx.x; e < nent; e += blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < (int)gridDim.x; ++k) acc += __ldcg(part + (size_t)k * nent + e);
        tot[e] = acc;
    }
    __syncthreads();
    // Σ_ab = Σ w θ_a θ_b - θ̄_a θ̄_b with θ̄ = Σ w θ / Σ w (gsl_stats_wmean)
    for (int e = threadIdx.x; e < p * (p + 1) / 2; e += blockDim.x) {
        int a = (int)((sqrt(8.0 * e + 1.0) - 1.0) * 0.5);
        while ((a + 1) * (a + 2) / 2 <= e) ++a;
        while (a * (a + 1) / 2 > e) --a;
        const int b = e - a * (a + 1) / 2;
        const double ma = tot[1 + a] / tot[0], mb = tot[1 + b] / tot[0];
        const double v = tot[1 + p + e] - ma * mb;
        sigma[a * p + b] = v;
        sigma[b * p + a] = v;
    }
}

// chol(scaling² Σ), lower triangle row-major (Metropolis.py:103-107).  One CTA,
// left-looking by columns in L itself: thread 0 forms the diagonal, then every
// thread forms one entry below it; each entry sums over k in increasing order, as
// the sequential Cholesky–Crout loop does.
__global__ void cholesky_kernel(int p, const double* __restrict__ sigma,
                                const double* __restrict__ scaling, double* __restrict__ L,
                                uint32_t* __restrict__ flags) {
    __shared__ double s_ljj;
    __shared__ int s_ok;
    const double s2 = (*scaling) * (*scaling);
    for (int k = threadIdx.x; k < p * p; k += blockDim.x) L[k] = s2 * sigma[k];
    if (threadIdx.x == 0) s_ok = 1;
    __syncthreads();
    for (int j = 0; j < p; ++j) {
        if (threadIdx.x == 0) {
            double d = L[j * p + j];
            for (int k = 0; k < j; ++k) d -= L[j * p + k] * L[j * p + k];
            if (!(d > 0.0)) {
                s_ok = 0;
            } else {
                s_ljj = sqrt(d);
                L[j * p + j] = s_ljj;
            }
        }
        __syncthreads();
        if (!s_ok) break;
        const double ljj = s_ljj;
        for (int i = j + 1 + threadIdx.x; i < p; i += blockDim.x) {
            double v = L[i * p + j];
            for (int k = 0; k < j; ++k) v -= L[i * p + k] * L[j * p + k];
            L[i * p + j] = v / ljj;
        }
        __syncthreads();
    }
    if (!s_ok) {
        // keep the walk defined: fall back to the scaled diagonal and report
        if (threadIdx.x == 0) raise_flag(flags, DEV_ERR_NOT_SPD);
        for (int k = threadIdx.x; k < p * p; k += blockDim.x) {
            const int i = k / p, c = k % p;
            L[k] = (i == c) ? sqrt(fmax(s2 * sigma[k], 0.0)) : 0.0;
        }
        return;
    }
    for (int k = threadIdx.x; k < p * p; k += blockDim.x)
        if (k % p > k / p) L[k] = 0.0;              // clear the upper triangle
}

// ---------------------------------------------------------------------------
// multinomial resampling (COV.py:160-251)
struct ResampleHdr {
    int total;        // number of copied rows (Σ counts)
    int first_src;    // source row of output row 0
    unsigned done;    // blocks of counts_rank_kernel finished
    int pad;
};

// sequential FP64 partial sums, as itertools.accumulate (COV.py:242-251)
// The additions stay strictly sequential (the reference's accumulation order, so the edges
// are bit-exact); one warp streams w through a shared-memory double buffer so that lane 0's
// chain of dependent additions never waits on global-memory latency.
constexpr int kCdfChunk = 1024;
__global__ void __launch_bounds__(32) cdf_kernel(const double* __restrict__ w, int n,
                                                 double* __restrict__ edges) {
    __shared__ double buf[2][kCdfChunk];
    if (blockIdx.x != 0) return;
    const int lane = threadIdx.x;
    const int nchunks = (n + kCdfChunk - 1) / kCdfChunk;
    auto load = [&](int c) {
        const int base = c * kCdfChunk;
        for (int k = lane; k < kCdfChunk; k += 32) buf[c & 1][k] = (base + k < n) ? w[base + k] : 0.0;
    };
    double acc = 0.0;
    if (lane == 0) edges[0] = 0.0;
    if (nchunks > 0) load(0);
    __syncwarp();
    for (int c = 0; c < nchunks; ++c) {
        if (c + 1 < nchunks) load(c + 1);            // the next chunk streams in meanwhile
        if (lane == 0) {
            const int base = c * kCdfChunk, len = min(kCdfChunk, n - base);
            const double* b = buf[c & 1];
            for (int k = 0; k < len; ++k) {
                acc += b[k];
                edges[base + k + 1] = acc;
            }
        }
        __syncwarp();
    }
}

// base[v] = Σ_{v' > v} v'·hist[v'] (reverse exclusive scan) then stable ranks within
// equal counts: start_i = base[c_i] + c_i · #{k < i : c_k = c_i}.  One CTA of 1024 threads.
constexpr int kRankCache = 4096;
__device__ void rank_counts(int n, const int* __restrict__ counts, int* __restrict__ hist, int* __restrict__ base,
                            int* __restrict__ seen, int* __restrict__ start, ResampleHdr* __restrict__ hdr) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    __shared__ int s_seen[kRankCache];
    if (threadIdx.x == 0) carry = 0;
    for (int k = threadIdx.x; k < kRankCache; k += blockDim.x) s_seen[k] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // values n .. 0 in chunks of blockDim, processed from high to low
    for (int top = n; top >= 0; top -= (int)blockDim.x) {
        const int v = top - (int)threadIdx.x;
        const int x = (v >= 1) ? v * __ldcg(hist + v) : 0;
        // inclusive scan inside the block in thread order (= decreasing v)
        int s = x;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane == 31) warp_tot[warp] = s;
        __syncthreads();
        if (warp == 0) {
            int wt = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, wt, o);
                if (lane >= o) wt += t;
            }
            warp_tot[lane] = wt;
        }
        __syncthreads();
        const int before = carry + (warp > 0 ? warp_tot[warp - 1] : 0) + s - x;
        if (v >= 0) base[v] = before;
        __syncthreads();
        if (threadIdx.x == 0) carry += warp_tot[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) hdr->total = carry;
    // stable ranks: warp 0 walks the chains in order
    if (warp != 0) return;
    int first = -1;
    for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        const int c = (i < n) ? __ldcg(counts + i) : 0;
        const unsigned peers = __match_any_sync(0xffffffffu, c);
        const int leader = __ffs(peers) - 1;
        const int rank = __popc(peers & ((1u << lane) - 1u));
        int old = 0;
        if (lane == leader && c > 0) {
            if (c < kRankCache) { old = s_seen[c]; s_seen[c] = old + __popc(peers); }
            else { old = seen[c]; seen[c] = old + __popc(peers); }
        }
        old = __shfl_sync(0xffffffffu, old, leader);
        if (c > 0) {
            const int st = base[c] + c * (old + rank);
            start[i] = st;
            if (st == 0) first = i;
        } else if (i < n) {
            start[i] = -1;
        }
        __syncwarp();
    }
    for (int o = 16; o > 0; o >>= 1) first = max(first, __shfl_xor_sync(0xffffffffu, first, o));
    if (lane == 0) hdr->first_src = first;
}

// counts[i] = #{j : edges[i] <= r_j < edges[i+1]}; r_j >= edges[n] dropped (gsl_histogram).
// One thread per uniform; the last block to finish (threadfence reduction: the block count is
// cleared before the launch) forms the histogram of the counts and the ranks.
__global__ void __launch_bounds__(1024) counts_rank_kernel(int n, uint64_t seed, const uint32_t* __restrict__ epoch,
                                                           const double* __restrict__ edges, int* __restrict__ counts,
                                                           int* __restrict__ hist, int* __restrict__ base,
                                                           int* __restrict__ seen, int* __restrict__ start,
                                                           ResampleHdr* __restrict__ hdr, unsigned* __restrict__ done) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) {
        u32x4 r = draw(seed, (uint32_t)j, 0u, STREAM_RESAMPLE, 0u, *epoch);
        const double x = u01_closed_open(r.x, r.y);
        if (x >= edges[0] && x < edges[n]) {
            // largest i with edges[i] <= x
            int lo = 0, hi = n;          // edges[lo] <= x < edges[hi]
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (x >= edges[mid]) lo = mid; else hi = mid;
            }
            atomicAdd(&counts[lo], 1);
        }
    }
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int c = __ldcg(counts + i);
        if (c > 0) atomicAdd(&hist[c], 1);
    }
    __threadfence_block();
    __syncthreads();
    rank_counts(n, counts, hist, base, seen, start, hdr);
}

__global__ void gather_kernel(int n, int p, const double* __restrict__ beta,
                              const int* __restrict__ counts, const int* __restrict__ start,
                              const ResampleHdr* __restrict__ hdr,
                              const double* __restrict__ th_in, const double* __restrict__ pr_in,
                              const double* __restrict__ da_in, double* __restrict__ th_out,
                              double* __restrict__ pr_out, double* __restrict__ da_out,
                              double* __restrict__ po_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double b = *beta;
    const int c = counts[i];
    if (c > 0) {
        const int s0 = start[i];
        for (int k = 0; k < c; ++k) {
            const int d = s0 + k;
            for (int j = 0; j < p; ++j) th_out[(size_t)d * p + j] = th_in[(size_t)i * p + j];
            pr_out[d] = pr_in[i];
            da_out[d] = da_in[i];
            po_out[d] = pr_in[i] + b * da_in[i];
        }
    }
    // rows left over when uniforms fell beyond the last edge repeat the first group's row
    const int d = i;
    if (d >= hdr->total && hdr->first_src >= 0) {
        const int src = hdr->first_src;
        for (int j = 0; j < p; ++j) th_out[(size_t)d * p + j] = th_in[(size_t)src * p + j];
        pr_out[d] = pr_in[src];
        da_out[d] = da_in[src];
        po_out[d] = pr_in[src] + b * da_in[src];
    }
}

// ---------------------------------------------------------------------------
// scaling adaptation (Metropolis.py:262-281); then a new epoch
__global__ void adapt_kernel(double aw, double rw, unsigned long long* __restrict__ counters,
                             double* __restrict__ scaling, uint32_t* __restrict__ epoch) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const double acc = (double)counters[0];
    const double tot = (double)(counters[0] + counters[1] + counters[2]);
    const double acceptance = tot > 0.0 ? acc / tot : 0.0;
    double kc = (aw * acceptance + rw) / (aw + rw);
    if (kc < 0.1) kc = 0.1;
    if (kc > 1.0) kc = 1.0;
    *scaling = kc;
    counters[0] = counters[1] = counters[2] = 0ull;
    *epoch += 1u;
}

}  // namespace ag

// ---------------------------------------------------------------------------
// C ABI
using namespace ag;

static inline int blocks(int n, int t) { return (n + t - 1) / t; }

static int check_state(const ag_stage_state* st) {
    AG_REQUIRE(st && st->beta && st->dbeta_cov && st->scaling && st->sigma && st->chol && st->w &&
                   st->counters && st->epoch && st->dev_flags,
               "stage state has a NULL member");
    AG_REQUIRE(st->chain0 >= 0, "stage state chain0 must be >= 0 (got %d)", st->chain0);
    return AG_OK;
}

extern "C" int ag_prior_sample(int32_t n, int32_t p, const double* lo, const double* hi,
                               uint64_t seed, uint32_t attempt, const uint32_t* redraw,
                               double* theta, void* stream) {
    AG_REQUIRE(n > 0 && p > 0 && lo && hi && theta, "invalid arguments");
    prior_sample_kernel<<<blocks(n, 256), 256, 0, as_stream(stream)>>>(n, p, lo, hi, seed, attempt,
                                                                        redraw, theta);
    return launch_status("prior_sample_kernel");
}

extern "C" int ag_prior_llk(const double* theta, int32_t n, int32_t p, const double* lo,
                            const double* hi, uint32_t* mask, double* prior, void* stream) {
    AG_REQUIRE(n > 0 && p > 0 && theta && lo && hi, "invalid arguments");
    prior_llk_kernel<<<blocks(n, 256), 256, 0, as_stream(stream)>>>(theta, n, p, lo, hi, mask, prior);
    return launch_status("prior_llk_kernel");
}

extern "C" int ag_propose(const ag_stage_state* st, const double* theta, int32_t n, int32_t p,
                          const double* lo, const double* hi, uint64_t seed, uint32_t step,
                          double* cand, uint32_t* mask, double* cprior, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && p > 0 && p <= kMaxPLarge && theta && lo && hi && cand && mask && cprior,
               "invalid arguments (p must be in 1..%d)", kMaxPLarge);
    cudaStream_t s = as_stream(stream);
    if (p <= kMaxP) {
        propose_kernel<<<blocks(n, 128), 128, 0, s>>>(theta, n, p, st->chol, lo, hi, seed, step, st->epoch, cand,
                                                       mask, cprior, st->chain0);
        return launch_status("propose_kernel");
    }
    const size_t smem = (size_t)kProposeWarps * p * sizeof(double);
    if (smem > 48 * 1024) {
        rc = cuda_status(cudaFuncSetAttribute(propose_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem),
                         "cudaFuncSetAttribute(propose_warp_kernel)");
        if (rc) return rc;
    }
    propose_warp_kernel<<<blocks(n, kProposeWarps), kProposeWarps * 32, smem, s>>>(
        theta, n, p, st->chol, lo, hi, seed, step, st->epoch, cand, mask, cprior, st->chain0);
    return launch_status("propose_warp_kernel");
}

extern "C" int ag_accept(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed,
                         uint32_t step, const uint32_t* mask, const double* cand,
                         const double* cprior, const double* cdata, double* theta, double* prior,
                         double* data, double* post, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && p > 0 && mask && cand && cprior && cdata && theta && prior && data && post,
               "invalid arguments");
    accept_kernel<<<blocks(n, 256), 256, 0, as_stream(stream)>>>(
        n, p, st->beta, seed, step, st->epoch, mask, cand, cprior, cdata, theta, prior, data, post,
        st->counters, st->chain0);
    return launch_status("accept_kernel");
}

extern "C" int ag_accept_floor(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step,
                               const uint32_t* mask, const double* cprior, const double* post, double* llk_floor,
                               void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && mask && cprior && post && llk_floor, "invalid arguments");
    accept_floor_kernel<<<blocks(n, 256), 256, 0, as_stream(stream)>>>(n, st->beta, seed, step, st->epoch, mask,
                                                                        cprior, post, llk_floor, st->chain0);
    return launch_status("accept_floor_kernel");
}

extern "C" int ag_posterior(const ag_stage_state* st, int32_t n, const double* prior,
                            const double* data, double* post, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && prior && data && post, "invalid arguments");
    posterior_kernel<<<blocks(n, 256), 256, 0, as_stream(stream)>>>(n, st->beta, prior, data, post);
    return launch_status("posterior_kernel");
}

// COV workspace: schedule state | grid barrier | partial moments (two round buffers of
// kGridPoints x chunks x 2, then the final chunks x 2)
static size_t cov_part_offset() { return (sizeof(CovState) + 255) / 256 * 256; }
static size_t cov_part_doubles(int n) { return (size_t)(2 * kGridPoints + 1) * blocks(n, kEvalChunk) * 2; }

extern "C" size_t ag_cov_workspace_bytes(int32_t n) {
    if (n <= 0) return 0;
    return cov_part_offset() + sizeof(GridBarrier) + cov_part_doubles(n) * sizeof(double);
}

// blocks of cov_schedule_kernel<BRENT> that fit on the current device at once (the cooperative
// launch's limit), looked up once per device
constexpr int kCoopMaxDevices = 64;
template <bool BRENT>
static int cov_coresident_blocks(int* out) {
    static std::mutex mu;
    static int cache[kCoopMaxDevices] = {};
    int dev = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kCoopMaxDevices)
        return set_error(AG_ERR_SIZE, "device %d is beyond the %d devices the COV schedule tracks", dev,
                         kCoopMaxDevices);
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        int occ = 0, sms = 0;
        rc = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, cov_schedule_kernel<BRENT>, 256, 0),
                         "cudaOccupancyMaxActiveBlocksPerMultiprocessor(cov_schedule_kernel)");
        if (rc) return rc;
        rc = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
                         "cudaDeviceGetAttribute(multiprocessor count)");
        if (rc) return rc;
        if (occ < 1) return set_error(AG_ERR_CUDA, "cov_schedule_kernel does not fit on an SM");
        cache[dev] = occ * sms;
    }
    *out = cache[dev];
    return AG_OK;
}

// median (one CTA), then the whole search and the weights in one cooperative launch; the
// caller's scratch holds the state, the barrier words and the partials
template <bool BRENT>
static int cov_schedule_launch(const ag_stage_state* st, const double* data_llk, int n, double target,
                               double tol, int maxiter, int rounds, void* scratch, cudaStream_t s) {
    char* base = static_cast<char*>(scratch);
    CovState* S = reinterpret_cast<CovState*>(base);
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(base + cov_part_offset());
    double* part = reinterpret_cast<double*>(base + cov_part_offset() + sizeof(GridBarrier));
    int grid = 0;
    int rc = cov_coresident_blocks<BRENT>(&grid);
    if (rc) return rc;
    const int items = kGridPoints * blocks(n, kEvalChunk);
    if (grid > items) grid = items;
    rc = cuda_status(cudaMemsetAsync(bar, 0, sizeof(GridBarrier), s), "cudaMemsetAsync(COV barrier)");
    if (rc) return rc;
    cov_median_kernel<<<1, 1024, 0, s>>>(data_llk, n, st->beta, S);
    rc = launch_status("cov_median_kernel");
    if (rc) return rc;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cuda_status(cudaLaunchKernelEx(&cfg, cov_schedule_kernel<BRENT>, data_llk, n, target, tol, maxiter,
                                          rounds, S, part, bar, st->beta, st->dbeta_cov, st->w, st->dev_flags),
                       "cov_schedule_kernel (cooperative launch)");
}

extern "C" int ag_cov_schedule(const ag_stage_state* st, const double* data_llk, int32_t n,
                               double target, double tol, void* workspace, size_t workspace_bytes,
                               void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 1 && data_llk, "invalid arguments (need at least two chains)");
    const size_t need = ag_cov_workspace_bytes(n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "ag_cov_schedule needs %zu bytes of 256-byte aligned workspace", need);
    // round 0 evaluates the full remaining step, rounds 1..kGridLevels one level each
    return cov_schedule_launch<false>(st, data_llk, n, target, tol, 0, kGridLevels + 1, workspace,
                                      as_stream(stream));
}

extern "C" int ag_cov_schedule_brent(const ag_stage_state* st, const double* data_llk, int32_t n,
                                     double target, double tol, int32_t maxiter, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 1 && data_llk && maxiter > 0, "invalid arguments");
    const size_t need = ag_cov_workspace_bytes(n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "ag_cov_schedule_brent needs %zu bytes of 256-byte aligned workspace", need);
    const int iters = maxiter < kBrentMaxIter ? maxiter : kBrentMaxIter;
    // round 0: the full step; round 1: the guess and the interior point; then one point per iteration
    return cov_schedule_launch<true>(st, data_llk, n, target, tol, iters, iters + 2, workspace,
                                     as_stream(stream));
}

static void sigma_grid(int n, int p, int* chunk, int* nblk, int* cpb) {
    *chunk = sigma_chunk(p);
    const int nchunks = blocks(n, *chunk);
    *cpb = blocks(nchunks, kSigmaBlocks);
    *nblk = blocks(nchunks, *cpb);
}

extern "C" size_t ag_sigma_workspace_bytes(int32_t n, int32_t p) {
    if (n <= 0 || p <= 0 || p > kMaxPLarge) return 0;
    int chunk, nblk, cpb;
    sigma_grid(n, p, &chunk, &nblk, &cpb);
    const size_t nent = 1 + p + (size_t)p * (p + 1) / 2;
    return ((size_t)nblk + 1) * nent * sizeof(double) + 256;    // partials, totals, the block count
}

extern "C" int ag_weighted_cov(const ag_stage_state* st, const double* theta, int32_t n, int32_t p,
                               void* workspace, size_t workspace_bytes, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && p > 0 && p <= kMaxPLarge && theta, "invalid arguments (p <= %d)", kMaxPLarge);
    const size_t need = ag_sigma_workspace_bytes(n, p);
    AG_REQUIRE(workspace && workspace_bytes >= need, "ag_weighted_cov needs %zu bytes", need);
    cudaStream_t s = as_stream(stream);
    int chunk, nblk, cpb;
    sigma_grid(n, p, &chunk, &nblk, &cpb);
    const int nent = 1 + p + p * (p + 1) / 2;
    const size_t smem = (size_t)chunk * (p + 1) * sizeof(double);
    if (smem > 48 * 1024) {
        rc = cuda_status(cudaFuncSetAttribute(sigma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "cudaFuncSetAttribute(sigma_kernel)");
        if (rc) return rc;
    }
    double* part = reinterpret_cast<double*>(workspace);
    double* tot = part + (size_t)nblk * nent;
    unsigned* done = reinterpret_cast<unsigned*>(tot + nent);
    rc = cuda_status(cudaMemsetAsync(done, 0, sizeof(unsigned), s), "cudaMemsetAsync(Σ block count)");
    if (rc) return rc;
    sigma_kernel<<<nblk, 256, smem, s>>>(theta, st->w, n, p, chunk, cpb, part, tot, done, st->sigma);
    return launch_status("sigma_kernel");
}

extern "C" int ag_cholesky_scaled(const ag_stage_state* st, int32_t p, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(p > 0 && p <= kMaxPLarge, "p must be in 1..%d", kMaxPLarge);
    cholesky_kernel<<<1, 256, 0, as_stream(stream)>>>(p, st->sigma, st->scaling, st->chol, st->dev_flags);
    return launch_status("cholesky_kernel");
}

// workspace layout: hdr (with the block count of counts_rank_kernel) | edges[n+1] |
// counts[n] (if not given) | hist[n+1] | base[n+1] | seen[n+1] | start[n]
static size_t align256(size_t b) { return (b + 255) / 256 * 256; }
extern "C" size_t ag_resample_workspace_bytes(int32_t n) {
    if (n <= 0) return 0;
    size_t b = align256(sizeof(ResampleHdr));
    b += align256((size_t)(n + 1) * sizeof(double));
    b += 5 * align256((size_t)(n + 1) * sizeof(int));
    return b;
}

extern "C" int ag_resample(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed,
                           const double* theta_in, const double* prior_in, const double* data_in,
                           double* theta_out, double* prior_out, double* data_out, double* post_out,
                           int32_t* counts, void* workspace, size_t workspace_bytes, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(n > 0 && p > 0 && theta_in && prior_in && data_in && theta_out && prior_out &&
                   data_out && post_out,
               "invalid arguments");
    AG_REQUIRE(theta_in != theta_out, "resampling is out of place: theta_in == theta_out");
    const size_t need = ag_resample_workspace_bytes(n);
    AG_REQUIRE(workspace && workspace_bytes >= need && aligned(workspace, 256),
               "ag_resample needs %zu bytes of 256-byte aligned workspace", need);
    cudaStream_t s = as_stream(stream);
    char* ws = static_cast<char*>(workspace);
    ResampleHdr* hdr = reinterpret_cast<ResampleHdr*>(ws);
    ws += align256(sizeof(ResampleHdr));
    double* edges = reinterpret_cast<double*>(ws);
    ws += align256((size_t)(n + 1) * sizeof(double));
    const size_t ib = align256((size_t)(n + 1) * sizeof(int));
    int* cnt_ws = reinterpret_cast<int*>(ws); ws += ib;
    int* hist = reinterpret_cast<int*>(ws); ws += ib;
    int* base = reinterpret_cast<int*>(ws); ws += ib;
    int* seen = reinterpret_cast<int*>(ws); ws += ib;
    int* start = reinterpret_cast<int*>(ws); ws += ib;
    int* cnt = counts ? counts : cnt_ws;
    rc = cuda_status(cudaMemsetAsync(cnt, 0, (size_t)n * sizeof(int), s), "memset counts");
    if (rc) return rc;
    rc = cuda_status(cudaMemsetAsync(hist, 0, (size_t)(n + 1) * sizeof(int), s), "memset hist");
    if (rc) return rc;
    rc = cuda_status(cudaMemsetAsync(seen, 0, (size_t)(n + 1) * sizeof(int), s), "memset seen");
    if (rc) return rc;
    rc = cuda_status(cudaMemsetAsync(&hdr->done, 0, sizeof(unsigned), s), "memset block count");
    if (rc) return rc;
    cdf_kernel<<<1, 32, 0, s>>>(st->w, n, edges);
    counts_rank_kernel<<<blocks(n, 1024), 1024, 0, s>>>(n, seed, st->epoch, edges, cnt, hist, base, seen, start,
                                                         hdr, &hdr->done);
    gather_kernel<<<blocks(n, 128), 128, 0, s>>>(n, p, st->beta, cnt, start, hdr, theta_in, prior_in,
                                                 data_in, theta_out, prior_out, data_out, post_out);
    return launch_status("resample kernels");
}

extern "C" int ag_adapt_scaling(const ag_stage_state* st, double aw, double rw, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    adapt_kernel<<<1, 32, 0, as_stream(stream)>>>(aw, rw, st->counters, st->scaling, st->epoch);
    return launch_status("adapt_kernel");
}

// ---------------------------------------------------------------------------
// Allocation-free COV β schedule.
//
// Some callers cannot call cudaMalloc when they run a stage: hosts whose
// device memory is entirely reserved up front by another allocator or by a
// fixed memory budget, embedders that must not change their device footprint
// after start-up, and loops that must not enter the allocator at all because
// cudaMalloc and cudaFree may synchronise the device.  This entry point
// needs no caller workspace: its scratch (the schedule state, the grid
// barrier words and the partial moments) lives in a file-scope device array of fixed
// size, reserved when this file's module is loaded on a device and held by
// every device that loads it until the process exits.  Under CUDA's default
// lazy module loading the module is loaded by the first use of any kernel or
// symbol of this file (the first call of this entry point, ag_cov_schedule,
// ag_resample, ...), which may then enter the driver's allocator once:
// callers make such a call during start-up.
//
// * Limit: n <= kNoAllocMaxChains chains; larger n is rejected.
// * All calls share the one array, and it keeps the last call's contents:
//   calls whose work overlaps on the GPU (different streams, or a call made
//   before the previous one finished on another stream) race on it; issue
//   them in order on one stream.
// * The first call on each device looks up the array's device address
//   (cudaGetSymbolAddress) with that device current; make that first call
//   before any stream capture.
namespace {

constexpr int32_t kNoAllocMaxChains = 1 << 18;
constexpr size_t kNoAllocState = (sizeof(CovState) + 255) / 256 * 256;
constexpr size_t kNoAllocBytes =
    kNoAllocState + sizeof(GridBarrier) +
    (size_t)(2 * kGridPoints + 1) * ((kNoAllocMaxChains + kEvalChunk - 1) / kEvalChunk) * 2 * sizeof(double);
static_assert(kNoAllocState == (sizeof(CovState) + 255) / 256 * 256, "no-alloc layout follows the workspace layout");
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_cov_scratch[kNoAllocBytes];

std::mutex g_scratch_mutex;
void* g_scratch_addr[kNoAllocMaxDevices] = {};

int scratch_address(void** out) {
    int dev = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return set_error(AG_ERR_SIZE, "device %d is beyond the %d devices this entry point tracks", dev,
                         kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        rc = cuda_status(cudaGetSymbolAddress(&p, g_cov_scratch), "cudaGetSymbolAddress(g_cov_scratch)");
        if (rc) return rc;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return AG_OK;
}

}  // namespace

extern "C" int32_t ag_cov_schedule_noalloc_max_chains(void) { return kNoAllocMaxChains; }

extern "C" int ag_cov_schedule_noalloc(const ag_stage_state* st, const double* data_llk, int32_t n,
                                       double target, double tol, void* stream) {
    int rc = check_state(st);
    if (rc) return rc;
    AG_REQUIRE(data_llk != nullptr, "data_llk is NULL");
    if (n < 2 || n > kNoAllocMaxChains)
        return set_error(AG_ERR_SIZE,
                         "ag_cov_schedule_noalloc supports 2 to %d chains (got %d); use ag_cov_schedule "
                         "with a caller workspace for more",
                         kNoAllocMaxChains, n);
    void* scratch = nullptr;
    rc = scratch_address(&scratch);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    // the state block starts from zero on every call; the partials are written before they are read
    rc = cuda_status(cudaMemsetAsync(scratch, 0, kNoAllocState, s), "cudaMemsetAsync(scratch state)");
    if (rc) return rc;
    return cov_schedule_launch<false>(st, data_llk, n, target, tol, 0, kGridLevels + 1, scratch, s);
}
