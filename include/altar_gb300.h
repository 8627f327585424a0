/*
 * altar_gb300: C ABI of the GB300 (sm_103a) CATMIP hot path.
 *
 * Every pointer argument is a DEVICE pointer owned by the caller unless the
 * comment says otherwise; the library allocates nothing and keeps no global
 * mutable state apart from a per-thread error string, with one exception:
 * ag_cov_schedule_noalloc keeps its scratch in a fixed device array inside the
 * library (about 95 KB per device) and caches that array's address per
 * device; the COV schedule entry points cache the co-resident block count of
 * their cooperative kernel per device.  Every call is
 * asynchronous on the given stream (a cudaStream_t passed as void*, NULL =
 * legacy default stream) and returns AG_OK or an error code; the message of
 * the last error of the calling thread is available from ag_last_error().
 *
 * Array layouts:
 *   theta    N x p row-major FP64 (chain-major), as the reference's θ
 *            (altar/altar/bayesian/CoolingStep.py:25)
 *   vectors  FP64 length-N prior / data / posterior log-likelihoods
 *   sigma    p x p row-major FP64; chol: lower-triangular p x p row-major
 */
#ifndef ALTAR_GB300_H
#define ALTAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define AG_OK 0
#define AG_ERR_ARG 1      /* invalid argument (null pointer, bad size, bad layout) */
#define AG_ERR_CUDA 2     /* a CUDA runtime call failed */
#define AG_ERR_DEVICE 3   /* a kernel raised a device flag (timeout, non-SPD pivot) */
#define AG_ERR_SIZE 4     /* a size exceeds what the entry point supports */

/* forward models */
#define AG_MODEL_MOGI 1
#define AG_MODEL_CDM 2

/* per-chain status bits written by the forward models and the proposal */
#define AG_CHAIN_OUT_OF_SUPPORT 1u  /* outside the prior support (Uniform.verify) */
#define AG_CHAIN_ABOVE_SURFACE 2u   /* CDM reaches above the free surface */
#define AG_CHAIN_NONFINITE 4u       /* non-finite log-likelihood */

/* device error flags (ag_stage_state.dev_flags) */
#define AG_DEV_ERR_TIMEOUT 1u
#define AG_DEV_ERR_NOT_SPD 2u

/* Station arrays: padded to a multiple of AG_STATION_TILE entries; padding
 * entries carry weight 0 and contribute nothing. */
#define AG_STATION_TILE 128

/*
 * Observation points of one or more concatenated datasets.
 * Replaces the per-source state the reference attaches through
 * libcudacdm.locations / los / data / oid (models/cdm/ext/cudacdm/source.cc:155,235,90,304)
 * and the Mogi equivalents (models/mogi/ext/cudamogi/source.cc).
 */
typedef struct ag_station_set {
    const float* xy;       /* [m_padded][4]: x_hi, x_lo, y_hi, y_lo; x = x_hi + x_lo (m) */
    const float* losd;     /* [m_padded][4]: LOS east, north, up; observed LOS displacement (m) */
    const float* weight;   /* [m_padded]: 1/σ² of each observation (diagonal Cd), 0 for padding */
    const int32_t* oid;    /* [m_padded]: dataset id, selects θ[offset_idx + oid]; NULL = none */
    int32_t m;             /* number of observations */
    int32_t m_padded;      /* multiple of AG_STATION_TILE */
    const float* tile_box; /* [m_padded / AG_STATION_TILE][4]: x min, x max, y min, y max of each tile's
                              observations, rounded outwards (ag_station_boxes); needed by the CDM,
                              which picks its quadrature per tile; NULL for Mogi */
    const int32_t* order;  /* [m_padded]: column of stored observation j in the caller's order, for the
                              residual rows (a permutation with order[j] = j for j >= m); NULL = the
                              stored order.  Storing the observations along a space-filling curve
                              makes the CDM's tiles compact: fewer quadrature nodes per station */
} ag_station_set;

/*
 * Fills tile_box from xy: the bounding box of each tile of AG_STATION_TILE
 * consecutive observations (padding left out), rounded outwards to FP32.  No
 * counterpart in the reference.  Observations ordered so that consecutive ones
 * lie close together (rows of a grid, a space-filling order) give small boxes
 * and let the CDM integrate more of its rectangles with few nodes.
 */
int ag_station_boxes(const float* xy, int32_t m, int32_t m_padded, float* tile_box, void* stream);

/*
 * Parameter layout of a sample row.  Replaces libcudacdm.layout
 * (models/cdm/ext/cudacdm/source.cc:378: xIdx, dIdx, openingIdx, aXIdx,
 * omegaXIdx, offsetIdx) and libcudamogi.layout
 * (models/mogi/ext/cudamogi/source.cc:378: xIdx, dIdx, sIdx, offsetIdx).
 */
typedef struct ag_layout {
    int32_t nparams;        /* row stride of θ (p) */
    int32_t x_idx;          /* east coordinate of the (first) source; north is x_idx + 1 */
    int32_t depth_idx;      /* depth, positive down (m) */
    int32_t strength_idx;   /* Mogi: volume change; CDM: opening (m) */
    int32_t axes_idx;       /* CDM: semi-axes ax, ay, az at axes_idx .. axes_idx + 2 */
    int32_t omega_idx;      /* CDM: clockwise rotations about x, y, z in degrees */
    int32_t offset_idx;     /* first per-dataset offset parameter; -1 = none */
    int32_t log_strength;   /* Mogi: 1 = θ holds log10(ΔV) as in the reference, 0 = ΔV */
    int32_t nsources;       /* Mogi: number of point sources (>= 1) */
    int32_t source_stride;  /* Mogi: parameter distance between consecutive sources */
    int32_t variant;        /* CDM kernel launch variant (0 = default; see ag_forward_variants) */
    int32_t reserved;
    double nu;              /* Poisson ratio */
} ag_layout;

/* number of launch variants of a forward model (autotuning candidates) */
int32_t ag_forward_variants(int model);

/* Last error message of the calling thread (NUL-terminated, truncated to len). */
int ag_last_error(char* buf, size_t len);

/* Library version string (static storage, host pointer). */
const char* ag_version(void);

/*
 * Bytes of caller-provided device workspace the forward model needs for n chains.
 */
size_t ag_forward_workspace_bytes(int model, int32_t n);

/*
 * Fused batched forward model + residual + diagonal-Cd whitening + FP64
 * per-chain data log-likelihood:
 *     llk[i] = norm - 1/2 * sum_j w_j * (u_j(θ_i) - d_j - θ_i[offset_idx + oid_j])^2
 * with u the LOS-projected Mogi (models/mogi/lib/libmogi/Source.cc:65-118) or
 * CDM (models/cdm/cdm/libcdm.py:39-247, cdm/Source.py:48-91) displacement.
 * Replaces libcudamogi.residuals / libcudacdm.residuals plus the per-chain
 * L2.withCovariance loop (models/cdm/cdm/CUDA.py:71-107, altar/altar/norms/L2.py:39-52)
 * for diagonal Cd.
 *   mask_in:    optional; chains with a non-zero word are skipped (llk untouched)
 *   chain_status: optional; receives AG_CHAIN_* bits (CDM geometry check)
 *   residuals:  optional N x m_padded FP32 residual rows (every station
 *               below m, whatever its weight; 0 in the padding)
 *   workspace:  ag_forward_workspace_bytes(model, n) bytes, 256-byte aligned
 */
int ag_forward_llk(int model, const ag_layout* layout, const double* theta, int32_t n,
                   const ag_station_set* stations, double norm, const uint32_t* mask_in,
                   double* llk, uint32_t* chain_status, float* residuals,
                   void* workspace, size_t workspace_bytes, void* stream);

/*
 * ag_forward_llk with early rejection (no counterpart in the reference): a chain whose
 * log-likelihood is found below llk_floor[i] (ag_accept_floor) part way through the
 * stations stops there and gets llk = -inf; every other chain's llk is exactly what
 * ag_forward_llk computes.  The Metropolis chains are then the same as without it, with
 * less work for the proposals that are rejected.  CDM: applied per tile of stations;
 * Mogi: the floor is ignored.  No residual rows.
 */
int ag_forward_llk_floor(int model, const ag_layout* layout, const double* theta, int32_t n,
                         const ag_station_set* stations, double norm, const uint32_t* mask_in,
                         const double* llk_floor, double* llk, uint32_t* chain_status,
                         void* workspace, size_t workspace_bytes, void* stream);

/*
 * ag_forward_llk restricted to the chains index[0 .. *count) (device-side
 * count, e.g. the survivors of a delayed-acceptance screen); llk, chain_status
 * and residual rows of the other chains are left untouched.  No counterpart in
 * the reference (its likelihood always evaluates every chain).
 */
int ag_forward_llk_subset(int model, const ag_layout* layout, const double* theta, int32_t n,
                          const ag_station_set* stations, double norm, const int32_t* index,
                          const int32_t* count, double* llk, uint32_t* chain_status,
                          float* residuals, void* workspace, size_t workspace_bytes, void* stream);

/* ag_forward_llk_subset with early rejection (as ag_forward_llk_floor, floors by chain index) */
int ag_forward_llk_subset_floor(int model, const ag_layout* layout, const double* theta, int32_t n,
                                const ag_station_set* stations, double norm, const int32_t* index,
                                const int32_t* count, const double* llk_floor, double* llk,
                                uint32_t* chain_status, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Work of the CDM likelihood kernel for each chain over the stations' m
 * observations: the FP32 operations (FMA = 2) and special-function operations
 * its plan executes, tile by tile (rectangles evaluated by their sides or by
 * quadrature nodes); 0 for chains above the free surface.  For roofline
 * accounting; sfu may be NULL.  No counterpart in the reference.
 */
int ag_cdm_work(const ag_layout* layout, const double* theta, int32_t n, const ag_station_set* stations,
                double* flop, double* sfu, void* stream);

/*
 * CDM geometry check only: chain_status[i] |= AG_CHAIN_ABOVE_SURFACE where a
 * corner of the CDM lies above the free surface (models/cdm/cdm/libcdm.py:219-224).
 */
int ag_cdm_check(const ag_layout* layout, const double* theta, int32_t n,
                 uint32_t* chain_status, void* stream);

/*
 * Initial sample from independent Uniform[lo_j, hi_j) priors
 * (altar/altar/distributions/Base.py:44-54 with Uniform.py), drawn from
 * Philox stream PRIOR at counter (chain, j, attempt).  Only rows whose
 * redraw[i] != 0 are drawn when redraw is non-NULL.
 */
int ag_prior_sample(int32_t n, int32_t p, const double* lo, const double* hi, uint64_t seed,
                    uint32_t attempt, const uint32_t* redraw, double* theta, void* stream);

/*
 * Uniform prior: mask[i] |= AG_CHAIN_OUT_OF_SUPPORT if some θ_ij is outside
 * [lo_j, hi_j] (altar/altar/distributions/Uniform.py:45-72) and
 * prior[i] = -sum_j log(hi_j - lo_j) (altar/altar/distributions/Base.py:61-79).
 */
int ag_prior_llk(const double* theta, int32_t n, int32_t p, const double* lo, const double* hi,
                 uint32_t* mask, double* prior, void* stream);

/*
 * Device-resident annealing state shared by the stage kernels.
 */
typedef struct ag_stage_state {
    double* beta;          /* [1] current β */
    double* dbeta_cov;     /* [2] last δβ and the COV it achieved */
    double* scaling;       /* [1] Metropolis proposal scaling */
    double* sigma;         /* [p*p] parameter covariance Σ */
    double* chol;          /* [p*p] lower Cholesky factor of scaling² Σ */
    double* w;             /* [N] normalised importance weights */
    unsigned long long* counters; /* [3] accepted, rejected, unlikely of the current stage */
    uint32_t* epoch;       /* [1] stage counter feeding the random streams */
    uint32_t* dev_flags;   /* [1] AG_DEV_ERR_* bits */
    int32_t chain0;        /* global index of the first chain these rows hold: the proposal and
                              accept streams are keyed by chain0 + row, so a population split
                              across ranks draws what one process would (0 = unsplit) */
    int32_t reserved;
} ag_stage_state;

/*
 * Metropolis proposal + Uniform verify + prior (altar/altar/bayesian/Metropolis.py:160-183,236-259):
 *   cand = θ + (L z)ᵀ, z ~ N(0, I) (Philox stream PROPOSAL, Box-Muller);
 *   rows outside the support are flagged in mask and replaced by θ;
 *   cprior = uniform log prior of cand.
 */
int ag_propose(const ag_stage_state* st, const double* theta, int32_t n, int32_t p,
               const double* lo, const double* hi, uint64_t seed, uint32_t step,
               double* cand, uint32_t* mask, double* cprior, void* stream);

/*
 * Metropolis accept/reject (altar/altar/bayesian/Metropolis.py:185-223):
 *   cpost = cprior + β cdata; rejected if mask, unlikely if log(u) > cpost - post
 *   (u ~ U(0,1], Philox stream ACCEPT), else θ, prior, data, post take the candidate's.
 *   Counters accumulate into st->counters.
 */
int ag_accept(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed, uint32_t step,
              const uint32_t* mask, const double* cand, const double* cprior, const double* cdata,
              double* theta, double* prior, double* data, double* post, void* stream);

/*
 * Early rejection (no counterpart in the reference, which evaluates every candidate in
 * full, Metropolis.py:186): llk_floor[i] = the data log-likelihood below which step
 * `step`'s proposal of chain i is certainly rejected by ag_accept with the same seed, step
 * and stage state, (post + log u − cprior)/β with the accept test's own uniform u, lowered
 * by a relative 1e-9; -inf for masked chains or β = 0.  Pass it to ag_forward_llk_floor
 * between ag_propose and ag_accept.
 */
int ag_accept_floor(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step,
                    const uint32_t* mask, const double* cprior, const double* post, double* llk_floor,
                    void* stream);

/*
 * Bytes of workspace ag_cov_schedule needs for n chains.
 */
size_t ag_cov_workspace_bytes(int32_t n);

/*
 * COV β schedule with the iterative grid solver
 * (altar/altar/bayesian/COV.py:91-102, Grid.py:48-59, altar/lib/libaltar/bayesian/COV.cc:222-368):
 * median of data llk, 11-point grid refinement of δβ until COV(w) hits
 * target within tol, β += δβ, w normalised importance weights at the final δβ.
 */
int ag_cov_schedule(const ag_stage_state* st, const double* data_llk, int32_t n,
                    double target, double tol, void* workspace, size_t workspace_bytes,
                    void* stream);

/*
 * δβ by Brent's minimiser (replaces altar.ext.altar.dbeta_brent,
 * altar/ext/dbeta.cc:39-96 → COV::dbeta_brent, COV.cc:58-219): minimises
 * (COV − target)² over [0, 1 − β] from the guess 5e-5, stops when the COV of
 * the latest point is within tol of the target or after maxiter iterations
 * (at most 128 run on the device), keeps the best point.  Same outputs and
 * workspace (ag_cov_workspace_bytes) as ag_cov_schedule.
 */
int ag_cov_schedule_brent(const ag_stage_state* st, const double* data_llk, int32_t n,
                          double target, double tol, int32_t maxiter, void* workspace,
                          size_t workspace_bytes, void* stream);

/*
 * Allocation-free variant of ag_cov_schedule (no counterpart in the reference).
 * For callers that cannot allocate device memory when they drive the schedule
 * (a fixed pre-reserved device budget, a device footprint that must not change
 * after start-up, or a loop that must not enter the allocator because cudaMalloc
 * and cudaFree may synchronise the device).  Same inputs and
 * results as ag_cov_schedule without the workspace: the scratch is a fixed
 * device array inside the library (about 95 KB, held by every device that
 * loads the library until exit).  Supports at most
 * ag_cov_schedule_noalloc_max_chains() chains (262,144); more returns
 * AG_ERR_SIZE.  All calls share that array: calls that overlap on the GPU
 * race, so issue them in order on one stream.  The first call on a device
 * looks up the array's address (and the schedule kernel's co-resident block
 * count) and should come before any stream capture.
 * The array is reserved when the library's stage module is loaded on a device:
 * under CUDA's default lazy module loading that happens at the first call into
 * any of the stage entry points (this one, ag_cov_schedule, ag_resample, ...),
 * which may then enter the driver's allocator once; make such a call during
 * start-up so that later calls allocate nothing.
 */
int ag_cov_schedule_noalloc(const ag_stage_state* st, const double* data_llk, int32_t n,
                            double target, double tol, void* stream);
int32_t ag_cov_schedule_noalloc_max_chains(void);

/* Bytes of workspace ag_weighted_cov needs. */
size_t ag_sigma_workspace_bytes(int32_t n, int32_t p);

/*
 * Weighted parameter covariance (altar/altar/bayesian/COV.py:106-156):
 * θ̄ = Σ w θ / Σ w, Σ = Σ w θ θᵀ - θ̄ θ̄ᵀ, into st->sigma.
 */
int ag_weighted_cov(const ag_stage_state* st, const double* theta, int32_t n, int32_t p,
                    void* workspace, size_t workspace_bytes, void* stream);

/*
 * chol = Cholesky(scaling² Σ) (altar/altar/bayesian/Metropolis.py:93-111);
 * a non-positive pivot raises AG_DEV_ERR_NOT_SPD in st->dev_flags.
 */
int ag_cholesky_scaled(const ag_stage_state* st, int32_t p, void* stream);

/* Bytes of workspace ag_resample needs. */
size_t ag_resample_workspace_bytes(int32_t n);

/*
 * Multinomial resampling (altar/altar/bayesian/COV.py:160-251):
 * edges = [0, cumsum(w)] accumulated sequentially in FP64, r_j ~ U[0,1)
 * (Philox stream RESAMPLE), counts[i] = #{j : edges_i <= r_j < edges_{i+1}}
 * (values >= the last edge are dropped, as gsl_histogram does), rows copied
 * in order of decreasing count (ties by increasing index), each count times;
 * rows left over when some r_j were dropped repeat the first copied row.
 * posterior_out = prior + β data.  counts (optional, N ints) receives the counts.
 */
int ag_resample(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed,
                const double* theta_in, const double* prior_in, const double* data_in,
                double* theta_out, double* prior_out, double* data_out, double* post_out,
                int32_t* counts, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Proposal scaling adaptation (altar/altar/bayesian/Metropolis.py:262-281):
 * kc = (aw·acc + rw)/(aw + rw) clamped to [0.1, 1], acc = accepted/total;
 * then clears the counters and advances the epoch.
 */
int ag_adapt_scaling(const ag_stage_state* st, double aw, double rw, void* stream);

/* posterior = prior + β data (altar/altar/models/Bayesian.py:105-115). */
int ag_posterior(const ag_stage_state* st, int32_t n, const double* prior, const double* data,
                 double* post, void* stream);

/* ---------------------------------------------------------------------------
 * Linear Gaussian model (models/linear/linear/Linear.py:152-185) with the data
 * covariance folded in: A = L⁻¹ G, b = L⁻¹ d for Cd = L Lᵀ, so that
 * llk = norm - 1/2 |A θ - b|² (the correct Gaussian form; the reference takes
 * norm - |L r|/2, Linear.py:182).
 */
typedef struct ag_linear_model {
    const double* a64;        /* [m_obs][p] FP64 A */
    const double* b64;        /* [m_obs] FP64 b */
    const uint16_t* a_split;  /* [m_obs][3 kpad] BF16 [A_hi | A_hi | A_lo] from ag_linear_prepare */
    int32_t m_obs;
    int32_t p;
} ag_linear_model;

/* p rounded up to the tensor-core K tile (64) */
int32_t ag_linear_kpad(int32_t p);
/* build the split BF16 operand of A (m x 3 kpad) */
int ag_linear_prepare(const double* A, int32_t m, int32_t p, uint16_t* a_split, void* stream);
/* workspace of ag_linear_llk for n chains */
size_t ag_linear_workspace_bytes(int32_t m, int32_t p, int32_t n);
/*
 * llk[i] = norm - 1/2 |A θ_i - b|² with A(θ - θ₀) on the tcgen05 tensor cores (split BF16,
 * FP32 accumulation) and ρ₀ = A θ₀ - b in FP64 (θ₀ = mean of the chains).  Replaces the
 * dgemm + per-chain norm loop of Linear.dataLikelihood.  flags receives AG_DEV_ERR_TIMEOUT.
 */
int ag_linear_llk(const ag_linear_model* model, const double* theta, int32_t n, double norm,
                  double* llk, void* workspace, size_t workspace_bytes, uint32_t* flags,
                  void* stream);
/* the same log-likelihood entirely in FP64 CUDA cores (reference path for checks) */
int ag_linear_llk_fp64(const ag_linear_model* model, const double* theta, int32_t n, double norm,
                       double* llk, void* stream);

/*
 * Dense-Cd whitening of one dataset's residual block (replaces the per-chain
 * L2.withCovariance dtrmv loop, altar/altar/norms/L2.py:39-52, for dense Cd):
 * llk[i] -= 1/2 |W (r_i - r̄) + W r̄|² over the block's columns, with W = L⁻¹
 * (Cd = L Lᵀ), r̄ the mean residual of up to 256 evenly spaced chains,
 * W (r - r̄) on the tcgen05 tensor cores (split BF16, FP32 accumulation) and
 * W r̄ in FP64.
 */
typedef struct ag_whiten_block {
    const double* w64;        /* [m][m] FP64 W = L⁻¹ */
    const uint16_t* w_split;  /* [m][3 kpad(m)] BF16 [W_hi | W_hi | W_lo] (ag_linear_prepare) */
    int32_t col0;             /* first column of the block in the residual rows */
    int32_t m;                /* observations in the block */
} ag_whiten_block;

size_t ag_whiten_workspace_bytes(int32_t m, int32_t n);
/* resid: n rows of ldr FP32 residuals (ag_forward_llk's residual output) */
int ag_whiten_llk(const ag_whiten_block* block, const float* resid, int32_t ldr, int32_t n, double* llk,
                  void* workspace, size_t workspace_bytes, uint32_t* flags, void* stream);

/* ---------------------------------------------------------------------------
 * Reverso two-reservoir magma model (FP64).  Replaces the libreverso capsule
 * module (models/reverso/ext/reverso/source.cc: newSource(G, v, mu, drho, g),
 * locations, data, layout(Qin, H_s, H_d, a_s, a_d, a_c indices), displacements,
 * residuals) and the per-sample norm loop of models/reverso/reverso/Fast.py:52-90.
 */
typedef struct ag_reverso_model {
    const double* txy;       /* [n_obs][3]: time (s), east, north (m) of each observation point */
    const double* d;         /* [n_obs][3]: observed displacement east, north, up (m) */
    const double* w;         /* [n_obs][3]: 1/σ² of each component (diagonal Cd); 0 drops it */
    int32_t n_obs;
    int32_t nparams;         /* row stride of θ */
    int32_t qin_idx, hs_idx, hd_idx, as_idx, ad_idx, ac_idx;   /* parameter positions */
    int32_t east_cos;        /* 1: u_E = u_r cos φ, u_N = u_r sin φ (reverso.cc:92-96, the default
                                strategy); 0: u_E = u_r sin φ, u_N = u_r cos φ (Native.py:96-100) */
    int32_t reserved;
    double G, v, mu, drho, g;  /* shear modulus, Poisson ratio, viscosity, density contrast, gravity */
} ag_reverso_model;

/*
 * llk[i] = norm - 1/2 Σ w (u - d)² over the 3 n_obs components of sample i; rows with
 * mask[i] != 0 are skipped (mask may be NULL).  predicted (NULL = none): n rows of the
 * 3 n_obs displacements (east, north, up per point), the reference's displacements().
 */
int ag_reverso_llk(const ag_reverso_model* model, const double* theta, int32_t n, double norm,
                   const uint32_t* mask, double* llk, double* predicted, void* stream);

/* ---------------------------------------------------------------------------
 * Learned surrogate and delayed acceptance.  No counterpart in the reference:
 * an MLP maps normalised source parameters to PCA coefficients of the LOS
 * field; it screens proposals (stage 1) before the exact model (stage 2).
 * Parameters: one FP32 buffer, per layer W (out x in, row-major) then b (out);
 * a BF16 copy of the same buffer feeds the products (FP32 accumulation).
 */
#define AG_MLP_MAX_LAYERS 8
typedef struct ag_mlp {
    int32_t nlayers;                        /* dense layers; GELU after all but the last */
    int32_t sizes[AG_MLP_MAX_LAYERS + 1];   /* input, hidden..., output widths */
} ag_mlp;

/* number of FP32 parameters (weights and biases) */
int64_t ag_mlp_param_count(const ag_mlp* net);
/* floats of activation storage ag_mlp_forward needs for n rows */
int64_t ag_mlp_activation_floats(const ag_mlp* net, int32_t n);
/* x = 2 (θ - lo)/(hi - lo) - 1 as FP32 (n x p) */
int ag_normalize_inputs(const double* theta, int32_t n, int32_t p, const double* lo,
                        const double* hi, float* x, void* stream);
/* out (n x sizes[nlayers]) = MLP(x); acts keeps pre- and post-activations for the backward pass */
int ag_mlp_forward(const ag_mlp* net, const float* params, const uint16_t* params_bf16,
                   const float* x, int32_t n, float* out, float* acts, void* stream);
/* gradients of the loss whose output gradient is dout (overwritten); scratch: 2 n max-width floats */
int ag_mlp_backward(const ag_mlp* net, const float* params, const uint16_t* params_bf16,
                    const float* x, int32_t n, const float* acts, float* dout, float* grads,
                    float* scratch, void* stream);
/* dout = (out - target)/n; row_loss[i] = 1/2 |out_i - target_i|² (optional) */
int ag_mse_grad(int32_t n, int32_t k, const float* out, const float* target, float* dout,
                float* row_loss, void* stream);
/* one Adam step (step number t >= 1) on the FP32 parameters; refreshes the BF16 copy if given */
int ag_adam_step(int64_t count, float* params, const float* grads, float* m, float* v, int32_t t,
                 float lr, float b1, float b2, float eps, uint16_t* params_bf16, void* stream);
/* BF16 copy of an FP32 buffer */
int ag_to_bf16(int64_t count, const float* src, uint16_t* dst, void* stream);
/*
 * Network forward on the tcgen05 tensor cores (layer widths after the input must be
 * multiples of 64).  Each layer is one persistent kernel: the activations as split BF16
 * rows [x_hi | x_lo] against the packed weights [W | W] (ag_mlp_tc_pack, from the BF16
 * copy), FP32 accumulation in TMEM, bias and GELU in the epilogue, which writes the next
 * layer's split input.  acts may be NULL (prediction only); otherwise it receives the FP32
 * pre-activations and outputs in ag_mlp_forward's layout.  workspace:
 * ag_mlp_tc_workspace_bytes(net, n) bytes, 256-byte aligned; flags: AG_DEV_ERR_TIMEOUT if
 * a bounded wait gave up.  No counterpart in the reference.
 */
size_t ag_mlp_tc_pack_bytes(const ag_mlp* net);
int ag_mlp_tc_pack(const ag_mlp* net, const uint16_t* wbf16, uint16_t* wpack, void* stream);
size_t ag_mlp_tc_workspace_bytes(const ag_mlp* net, int32_t n);
int ag_mlp_forward_tc(const ag_mlp* net, const float* params, const uint16_t* wpack, const float* x, int32_t n,
                      float* out, float* acts, void* workspace, size_t workspace_bytes, uint32_t* flags,
                      void* stream);
/* llk = norm - 1/2 (q0 - 2 hᵀ c̃ + c̃ᵀ G c̃) with c̃ = scale ⊙ coeff (n x k, k <= 96) */
int ag_surrogate_llk(int32_t n, int32_t k, const float* coeff, const float* scale, const float* gram,
                     const float* h, double q0, double norm, double* llk, void* stream);
/* delayed-acceptance stage 1 (Christen & Fox 2005): surrogate Metropolis test; survivors are
 * listed in index[0 .. *count) */
int ag_da_screen(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step,
                 const uint32_t* mask, const double* cprior, const double* csur, const double* prior,
                 const double* sur, int32_t* pass, int32_t* index, int32_t* count, void* stream);
/* delayed-acceptance stage 2: exact correction of the survivors; counters as ag_accept,
 * *screened (optional) counts the survivors */
int ag_da_accept(const ag_stage_state* st, int32_t n, int32_t p, uint64_t seed, uint32_t step,
                 const uint32_t* mask, const int32_t* pass, const double* cand, const double* cprior,
                 const double* cdata, const double* csur, double* theta, double* prior, double* data,
                 double* post, double* sur, unsigned long long* screened, void* stream);
/* early rejection of the stage-2 correction: llk_floor[i] = the exact log-likelihood below which
 * ag_da_accept with the same arguments certainly rejects chain i (-inf where it evaluates none);
 * for ag_forward_llk_subset_floor */
int ag_da_floor(const ag_stage_state* st, int32_t n, uint64_t seed, uint32_t step, const uint32_t* mask,
                const int32_t* pass, const double* cprior, const double* csur, const double* prior,
                const double* sur, const double* post, double* llk_floor, void* stream);

/* surrogate-transition variant: pass[i] = 1 where the surrogate chain θ_s moved away from θ;
 * those chains are listed in index[0 .. *count) for the exact correction (ag_da_accept with
 * θ_s as the candidate) */
int ag_da_moved(int32_t n, int32_t p, const double* theta, const double* theta_s, int32_t* pass,
                int32_t* index, int32_t* count, void* stream);

/* CUDA graph capture of a sequence of calls on one stream. */
int ag_graph_begin(void* stream);
int ag_graph_end(void* stream, void** graph_exec);
int ag_graph_launch(void* graph_exec, void* stream);
int ag_graph_destroy(void* graph_exec);

#ifdef __cplusplus
}
#endif

#endif /* ALTAR_GB300_H */
