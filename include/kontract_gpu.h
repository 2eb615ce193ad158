/*
 * kontract_gpu.h — C ABI of the GB300 (sm_103a) Monte-Carlo engine for the
 * compiled-contract pricing path of the `kontract` contract algebra.
 *
 * This is the drop-in boundary. A Rust crate (or any FFI) that today calls the
 * reference's pricer binds these symbols instead; every entry point below names
 * the reference interface it replaces (file:line in LePhilippeDucTai/kontracts).
 *
 * Conventions
 *  - Plain C types only: pointers, sizes, POD structs. No torch or CUDA types.
 *  - The caller owns every input and output buffer. `kx_program` is an opaque
 *    handle created by kx_compile and released by kx_program_free.
 *  - Device memory, streams and kernels belong to one lazily created
 *    per-process context (first GPU call). Calls are serialised on it by a
 *    mutex, so the API is thread-safe; it is not re-entrant from callbacks.
 *  - Every function returns kx_status. Nothing aborts. On failure the message
 *    of the calling thread is available from kx_last_error_message().
 *  - There is no CPU fallback: without a usable CUDA device the pricing entry
 *    points return KX_NO_DEVICE.
 */
#ifndef KONTRACT_GPU_H
#define KONTRACT_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KX_ABI_VERSION 1

/* Status codes. 1..7 mirror the seven variants of KontractError
 * (src/error.rs:6-28) one to one; Python raises ValueError for all of them,
 * as the reference binding does (src/bindings.rs:50-52). */
typedef enum kx_status {
    KX_OK = 0,
    KX_UNKNOWN_ASSET = 1,       /* KontractError::UnknownAsset      error.rs:8  */
    KX_TIME_OUT_OF_RANGE = 2,   /* KontractError::TimeOutOfRange    error.rs:11 */
    KX_STEP_OUT_OF_RANGE = 3,   /* KontractError::StepOutOfRange    error.rs:14 */
    KX_INCONSISTENT_PATH = 4,   /* KontractError::InconsistentPath  error.rs:17 */
    KX_SERDE = 5,               /* KontractError::Serde             error.rs:20 */
    KX_MALFORMED_CONTRACT = 6,  /* KontractError::MalformedContract error.rs:23 */
    KX_UNSUPPORTED = 7,         /* KontractError::Unsupported       error.rs:26 */
    KX_INVALID_ARGUMENT = 8,    /* null pointer, size or option out of range */
    KX_CUDA_ERROR = 9,          /* a CUDA runtime call failed */
    KX_DEVICE_TIMEOUT = 10,     /* a bounded device-side wait gave up */
    KX_NO_DEVICE = 11           /* no CUDA device could be used */
} kx_status;

typedef struct kx_program kx_program; /* compiled + lowered contract (opaque) */

/* ---- models --------------------------------------------------------------
 * Mirrors Gbm (src/simulator.rs:188-199) and HestonSimulator
 * (src/simulator.rs:453-471). `asset` is the name the contract's Spot(...)
 * observables must use (Simulator::asset_name, simulator.rs:98). */
enum { KX_MODEL_GBM = 0, KX_MODEL_HESTON = 1, KX_MODEL_MULTI_GBM = 2 /* kx_multi_gbm only */ };

/* Heston discretisation. REFERENCE_FLOOR is the reference's scheme
 * (Euler step, then v = max(v, 0); simulator.rs:517-534) and is the default.
 * FULL_TRUNCATION is Lord et al. (2010): drift and diffusion use max(v, 0)
 * and v itself is not floored. */
enum { KX_HESTON_REFERENCE_FLOOR = 0, KX_HESTON_FULL_TRUNCATION = 1 };

typedef struct kx_model {
    int32_t kind;          /* KX_MODEL_* */
    int32_t heston_scheme; /* KX_HESTON_*; ignored for GBM */
    double s0;             /* initial spot */
    double mu;             /* GBM drift (risk neutral: r - q) */
    double sigma;          /* GBM volatility */
    double v0, kappa, theta, sigma_v, rho; /* Heston parameters */
    double r;              /* Heston drift (risk-neutral rate) */
    const char *asset;     /* NUL-terminated asset name; NULL means "ASSET" */
} kx_model;

/* ---- Monte-Carlo configuration -------------------------------------------
 * Mirrors McConfig (src/pricer.rs:30-54): n_paths, seed, steps_per_year,
 * rate. The remaining fields select engine options the reference does not
 * have. */
enum { KX_RNG_PHILOX = 0, KX_RNG_SHARED_DRAWS = 1 };
/* Path arithmetic. FP32: paths in FP32, payoffs and their sums in FP64.
 * FP64: everything in FP64. FP32_KAHAN (kx_price; elsewhere it is FP32):
 * paths in FP32, and the sum over paths accumulated in Kahan-compensated FP32
 * (each path's value rounded to FP32 once, compensated sums per thread,
 * float-float across threads), FP64 only for the final merge of the chunk
 * statistics. */
enum { KX_PREC_FP32 = 0, KX_PREC_FP64 = 1, KX_PREC_FP32_KAHAN = 2 };

typedef struct kx_mc_config {
    uint64_t n_paths;        /* number of paths (0 gives a zero result) */
    uint64_t seed;           /* Philox key */
    uint32_t steps_per_year; /* fine-grid resolution (compiler.rs:54-65) */
    int32_t rng;             /* KX_RNG_*: Philox in registers, or the host normals
                                registered with kx_set_shared_draws */
    int32_t precision;       /* KX_PREC_*: path arithmetic type and payoff sums */
    int32_t flags;           /* KX_VR_* bits (kx_price only), else 0 */
    double rate;             /* deterministic discount rate */
} kx_mc_config;

/* Variance reduction of kx_price (McConfig.variance_reduction,
 * src/pricer.rs:108-230, src/variance_reduction.rs:60-235):
 * KX_VR_ANTITHETIC: GBM models price n_paths / 2 pairs (the paths of the
 * stream and their mirrors with negated normals), each pair valued at the mean
 * of its two PVs; other models price the plain paths.
 * KX_VR_CONTROL_VARIATE: the at-the-money call on the model's asset paid at
 * the grid's last date is the control, its Black-Scholes value (s0, sigma of
 * a GBM model; 100 and 0.2 otherwise, as the reference) known: per path
 * pv - (pv_call - bs); with KX_VR_ANTITHETIC the correction is applied to the
 * pair-averaged prices, and the standard error is the target's sample std over
 * sqrt(2 n_half) (pricer.rs:185-219). */
#define KX_VR_ANTITHETIC 1
#define KX_VR_CONTROL_VARIATE 2

/* Mirrors PriceResult (src/pricer.rs:58-71). */
typedef struct kx_price_result {
    double price;      /* mean discounted payoff */
    double sample_std; /* unbiased sample standard deviation of per-path PVs */
    double std_error;  /* sample_std / sqrt(n) */
    double ci95_low;   /* price - 1.959963984540054 * std_error */
    double ci95_high;  /* price + 1.959963984540054 * std_error */
    uint64_t n_paths;
} kx_price_result;

/* Mirrors BumpSizes (src/greeks.rs:22-39). With `relative` = 0 the bumps are
 * absolute (reference defaults spot 1e-2, vol 1e-2, rate 1e-4); with
 * `relative` = 1 each bump is multiplied by the bumped parameter's value. */
typedef struct kx_bumps {
    double spot, vol, rate;
    int32_t relative;
    int32_t smooth;        /* 1: reprice the barrier-smoothed payoff (see kx_adjoint_cfg) */
    double smoothing_width;/* log-space logistic width when smooth = 1 */
} kx_bumps;

/* Mirrors Greeks (src/greeks.rs:43-54), plus the standard error of each CRN
 * estimator (per-path finite differences). */
typedef struct kx_greeks {
    double price, delta, gamma, vega, rho;
    double price_se, delta_se, gamma_se, vega_se, rho_se;
} kx_greeks;

/* Pathwise-adjoint configuration (no reference counterpart). */
typedef struct kx_adjoint_cfg {
    uint32_t checkpoint_every; /* reverse sweep recomputes segments of this many steps */
    int32_t reserved;
    double smoothing_width;    /* log-space width w of the logistic barrier indicator;
                                  <= 0 selects 0.5 * sigma_eff * sqrt(dt) */
} kx_adjoint_cfg;

/* Sensitivities of the (smoothed) price. For GBM: d/ds0, d/dsigma, d/dr
 * (r moves drift and discount together, as greeks.rs:70 does). For Heston the
 * model parameters are filled as well. Each value has its standard error. */
typedef struct kx_sens {
    double price, price_se;
    double d_s0, d_sigma, d_r;
    double d_v0, d_kappa, d_theta, d_sigma_v, d_rho;
    double se_s0, se_sigma, se_r;
    double se_v0, se_kappa, se_theta, se_sigma_v, se_rho;
    double smoothing_width; /* the width actually used */
} kx_sens;

/* Timing and counters of the last pricing call on the calling process. */
typedef struct kx_launch_stats {
    double kernel_ms;          /* CUDA-event time of the main path kernel(s) */
    double reduce_ms;          /* CUDA-event time of the reduction kernels */
    double total_ms;           /* wall time of the whole call */
    uint64_t path_steps;       /* nominal path-steps (n_paths * grid steps) */
    uint64_t steps_simulated;  /* steps actually simulated (early exit skips) */
    uint32_t kernel_launches;  /* kernels launched by the call */
    uint32_t grid_blocks;
    uint32_t block_threads;
    uint32_t path_kernel;      /* last path kernel: 0 none, 1 k_paths (every
                                  contract), 2 k_lean (barrier/time contracts),
                                  3 k_lean on compiled static schedules, 4 the
                                  same with a running average of the spot,
                                  5 k_multi_lean (correlated factors, affine
                                  conditions and amounts), 6 k_mlmc_pairs
                                  (fine and coarse multilevel paths at once) */
    uint64_t h2d_bytes, d2h_bytes;
} kx_launch_stats;

/* Static plan of a contract: Plan (src/compiler.rs:25-34). */
typedef struct kx_plan_info {
    uint32_t n_assets;
    uint32_t n_fixed_dates;
    double horizon;
    int32_t needs_fine_grid;
    int32_t n_triggers;   /* lowered when/anytime/until slots */
    int32_t n_flows;      /* lowered one(...) leaves */
    int32_t n_accumulators;
} kx_plan_info;

/* ---- entry points ----------------------------------------------------------*/

/* ABI version of the loaded library (KX_ABI_VERSION). */
int32_t kx_abi_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char *kx_last_error_message(void);

/* Payload of the last failing call on this thread, so that a binding can
 * rebuild KontractError::TimeOutOfRange(f64) and StepOutOfRange(usize)
 * (src/error.rs:11-15) without parsing the message: *time receives the date
 * of KX_TIME_OUT_OF_RANGE (NaN for any other outcome), *step the index of
 * KX_STEP_OUT_OF_RANGE (UINT64_MAX otherwise). Either pointer may be NULL. */
kx_status kx_last_error_payload(double *time, uint64_t *step);

/* Parse the serde JSON of a Contract (Contract::from_json, src/ast.rs:215),
 * run the compiler (compile, src/compiler.rs:69) and lower the AST to the
 * flat trigger/flow/accumulator table the kernels interpret. Replaces the
 * per-call compile() inside price_gbm (src/pricer.rs:102). Host only. */
kx_status kx_compile(const char *contract_json, kx_program **out);
void kx_program_free(kx_program *prog);

/* Plan::assets / fixed_dates / horizon / needs_fine_grid (compiler.rs:25-34).
 * `assets_buf` receives the sorted asset names separated by '\n'. Host only. */
kx_status kx_program_plan(const kx_program *prog, kx_plan_info *info,
                          double *fixed_dates, size_t dates_cap,
                          char *assets_buf, size_t assets_cap);

/* Plan::time_grid_forced (src/compiler.rs:54-65). Writes at most `cap`
 * points, stores the full count in *n. Host only. */
kx_status kx_time_grid(const kx_program *prog, uint32_t steps_per_year,
                       int32_t force_fine, double *out, size_t cap, size_t *n);

/* Register host normals for KX_RNG_SHARED_DRAWS (path-major:
 * z[path * draws_per_path + d]; GBM uses draw k-1 at grid step k, Heston
 * draws 2(k-1) and 2(k-1)+1). The data is copied to the device. Exactly one
 * of z64 / z32 must be non-NULL. No reference counterpart (the reference
 * draws ChaCha8 normals inside Gbm::simulate, simulator.rs:233-241). */
kx_status kx_set_shared_draws(const double *z64, const float *z32,
                              uint64_t n_paths, uint64_t draws_per_path);
kx_status kx_clear_shared_draws(void);

/* price_gbm (src/pricer.rs:97-115): compile-time plan + grid, simulate, value
 * every path, summarise. `per_path_pv` (nullable, n_paths doubles) receives
 * the discounted value of every path (present_value, pricer.rs:344-355). */
kx_status kx_price(const kx_program *prog, const kx_model *model,
                   const kx_mc_config *cfg, kx_price_result *out,
                   double *per_path_pv);

/* ---- path ranges (sharding a price over GPUs or calls) --------------------
 * No reference counterpart. kx_price_chunks prices paths first_path ..
 * first_path + cfg->n_paths - 1 of the stream `cfg->seed` (the same paths a
 * kx_price of first_path + n_paths paths would simulate) and returns their
 * statistics per chunk of KX_STATS_CHUNK paths. first_path must be a multiple
 * of KX_STATS_CHUNK and first_path + n_paths at most 2^32; Philox only.
 * kx_merge_chunks merges chunk statistics in the given order (Chan et al.)
 * into a price: the chunks of consecutive ranges, merged in path order, give
 * exactly kx_price's result for the whole range. */
#define KX_STATS_CHUNK 16384u
typedef struct kx_chunk_stats {
    double n, mean, m2;  /* paths, mean, sum of squared deviations */
} kx_chunk_stats;
kx_status kx_price_chunks(const kx_program *prog, const kx_model *model,
                          const kx_mc_config *cfg, uint64_t first_path,
                          kx_chunk_stats *out, size_t cap, size_t *n_out);
kx_status kx_merge_chunks(const kx_chunk_stats *chunks, size_t n,
                          kx_price_result *out);
/* The statistics of one chunk of n <= KX_STATS_CHUNK values (values[i], or
 * values[i] - subtrahend[i] rounded to double when subtrahend is not NULL, as
 * a multilevel difference), on the host, bit for bit as the device reduction
 * computes them for finite values: exact integer sums of the values in units
 * of 2^-2 of the last mantissa bit of the chunk's largest value, one or two
 * roundings for the mean and for M2. */
kx_status kx_chunk_moments(const double *values, const double *subtrahend,
                           uint32_t n, kx_chunk_stats *out);

/* kx_price for callers that must not allocate device memory while pricing
 * (no counterpart in the reference). Same arguments and same result as
 * kx_price; every device buffer of the call lives in one static device array
 * of fixed size (about 9 MiB), so the call itself allocates nothing.
 * Limits: n_paths <= KX_FIXED_MAX_PATHS, time grid <= KX_FIXED_MAX_POINTS
 * points, cfg->rng == KX_RNG_PHILOX; otherwise KX_INVALID_ARGUMENT and nothing
 * runs. The first call of a process does the set-up (device made current,
 * address of the array looked up, library stream created): make it before
 * any stream capture. The address looked up is that of the array's copy on
 * the library's device (device 0 of the process, as for every entry point
 * here); it stays bound to that device for the life of the process. The
 * array is shared by all calls of the process, so calls are serialised by
 * the library lock; the call returns when its results are on the host. */
#define KX_FIXED_MAX_PATHS 1048576u
#define KX_FIXED_MAX_POINTS 8192u
kx_status kx_price_fixed_scratch(const kx_program *prog, const kx_model *model,
                                 const kx_mc_config *cfg, kx_price_result *out,
                                 double *per_path_pv);

/* price_batch_gbm (src/pricer.rs:250-294): one shared simulation on the
 * merged grid of all contracts, each contract valued on the same paths. */
kx_status kx_price_batch_shared(size_t n, const kx_program *const *progs,
                                const kx_model *model, const kx_mc_config *cfg,
                                kx_price_result *out);

/* kx_price_batch_shared with pathwise sensitivities (no reference
 * counterpart; the adjoint of greeks.rs:60-98's quantities on the shared
 * simulation): for a book whose contracts each pay one call, put or constant
 * amount at a fixed date (Europeans), the derivatives of the log-spot and of
 * the variance in every model parameter are carried forward along the shared
 * paths, and each contract's sensitivities are its payoff's derivative times
 * them at its date: d/ds0, d/dr (drift and discount together) and GBM
 * d/dsigma or Heston d/dv0, d/dkappa, d/dtheta, d/dsigma_v, d/drho, each with
 * its standard error; out[i] and sens[i].price are the prices of
 * kx_price_batch_shared. The derivatives are the pathwise ones of
 * kx_greeks_adjoint on the same paths (one forward pass for the whole book
 * instead of a reverse sweep per contract). Other contracts: KX_UNSUPPORTED
 * (kx_price_portfolio values any book with sensitivities). */
kx_status kx_price_batch_sens(size_t n, const kx_program *const *progs,
                              const kx_model *model, const kx_mc_config *cfg,
                              kx_price_result *out, kx_sens *sens);

/* Uneven portfolio in one persistent launch over a (contract, path-block)
 * work queue: each contract has its own model and config (its own grid,
 * n_paths and seed). Optional per-contract pathwise delta / vega (`sens`,
 * nullable: price, d_s0 and d_sigma filled). No reference counterpart: the
 * reference prices such a book with one price_gbm call per contract. */
kx_status kx_price_portfolio(size_t n, const kx_program *const *progs,
                             const kx_model *models, const kx_mc_config *cfgs,
                             kx_price_result *out, kx_sens *sens);

/* greeks_gbm (src/greeks.rs:60-98): CRN bump-and-reprice. The seven
 * reprices are plain jobs of one path launch, each priced as kx_price prices
 * the bumped model (the lean kernels), all on the seed's normals; the
 * estimators are means of per-path central differences. With bumps->smooth
 * one job carries the seven scenarios of the barrier-smoothed payoff. GBM
 * only (model->kind must be KX_MODEL_GBM); drift = rate, as the reference
 * rebuilds the model with Gbm::new(asset, s0, rate, sigma) (greeks.rs:70). */
kx_status kx_greeks_bump(const kx_program *prog, const kx_model *model,
                         const kx_mc_config *cfg, const kx_bumps *bumps,
                         kx_greeks *out);

/* greek_surface (src/surface.rs:104-137): greeks_gbm at every cell of the
 * grid spots x vols, out[i * n_vols + j] for spots[i], vols[j] (row-major as
 * GreekSurface, surface.rs:17-35; rho and the standard errors come along).
 * Every cell reprices with the same seed, so all cells and their seven bump
 * reprices value the same normals: the 7 x n_spots x n_vols reprices run as
 * the plain jobs of one path launch (several when the per-path values would
 * exceed 8 GiB), each cell bitwise equal to kx_greeks_bump at that cell. An
 * empty grid is KX_INCONSISTENT_PATH (surface.rs:113-117). */
kx_status kx_greek_surface(const kx_program *prog, const char *asset, const double *spots, size_t n_spots,
                           const double *vols, size_t n_vols, const kx_mc_config *cfg, const kx_bumps *bumps,
                           kx_greeks *out);

/* gbm_prices (src/calibration.rs:72-90) for several volatilities at once:
 * out[k * n_quotes + i] = price_gbm of the contract under
 * Gbm::new(asset, spots[i], cfg->rate, sigmas[k]) with cfg, NaN where that
 * price fails (calibration.rs:86). All n_sigmas x n_quotes prices come from
 * one path launch on the seed's normals (the common random numbers of the
 * reference's calibration, seed 42). Philox only. */
kx_status kx_calib_gbm_prices(const kx_program *prog, const char *asset, const double *spots, size_t n_quotes,
                              const double *sigmas, size_t n_sigmas, const kx_mc_config *cfg, double *out);

/* eval_obj_heston (src/calibration.rs:103-126) for a population of parameter
 * vectors params[k] = (v0, kappa, theta, sigma_v, rho) (5 doubles each):
 * obj[k] = sum over the quotes whose price succeeds of (price - quote)^2,
 * divided by n_quotes, with quotes[i] = (spot, market price) and the model
 * HestonSimulator::new(asset, spot, v0, kappa, theta, sigma_v, rho,
 * cfg->rate) (reference floor scheme). `prices` (nullable) receives the
 * n_params x n_quotes prices, NaN where one fails. One path launch prices the
 * whole population (a CMA-ES generation) on the seed's normals. */
kx_status kx_calib_heston_objective(const kx_program *prog, const char *asset, const double *quotes, size_t n_quotes,
                                    const double *params, size_t n_params, const kx_mc_config *cfg, double *obj,
                                    double *prices);

/* ---- correlated multi-factor GBM ------------------------------------------
 * Mirrors CorrelatedGbmN (src/multi_asset.rs:49-105) with its GbmFactor list
 * (src/fx.rs:149-169): n_assets >= 2 named factors (s0, mu, sigma) and their
 * n x n correlation, row-major in corr[i * n_assets + j]. */
#define KX_MAX_ASSETS 7
typedef struct kx_multi_gbm {
    uint32_t n_assets;
    uint32_t reserved;
    const char *names[KX_MAX_ASSETS];
    double s0[KX_MAX_ASSETS], mu[KX_MAX_ASSETS], sigma[KX_MAX_ASSETS];
    double corr[KX_MAX_ASSETS * KX_MAX_ASSETS];
} kx_multi_gbm;

/* price_gbm (src/pricer.rs:97) under a CorrelatedGbmN: every Spot(name) of the
 * contract reads its factor; each grid step draws n_assets normals, correlates
 * them with the lower Cholesky factor (numerics.rs:158-183) and steps every
 * factor exactly in log space (multi_asset.rs:85-170). Contracts whose price
 * conditions and amounts are affine in the spots (baskets, spreads) on a
 * time-only schedule run on the compiled kernel (path_kernel 5; Philox only),
 * the others on the general path kernel (M_MULTI). Fewer than 2 factors or a
 * negative volatility is KX_MALFORMED_CONTRACT, a spot of no factor
 * KX_UNKNOWN_ASSET. */
kx_status kx_price_multi(const kx_program *prog, const kx_multi_gbm *model, const kx_mc_config *cfg,
                         kx_price_result *out, double *per_path_pv);

/* ---- multilevel Monte Carlo ----------------------------------------------
 * Mirrors MlmcConfig (src/mlmc.rs:50-72; defaults n_levels 6, pilot_paths
 * 2000, target_variance 1e-4, cost_per_step 1) and MlmcResult (:75-96). */
#define KX_MLMC_MAX_LEVELS 20
typedef struct kx_mlmc_cfg {
    uint32_t n_levels;       /* finest level L: levels 0..L, level l has 2^l steps */
    uint32_t cost_per_step;
    uint64_t pilot_paths;
    double target_variance;
} kx_mlmc_cfg;

typedef struct kx_mlmc_result {
    kx_price_result price;
    uint32_t n_levels;       /* levels 0..n_levels are filled */
    uint32_t reserved;
    double level_means[KX_MLMC_MAX_LEVELS + 1];
    double level_variances[KX_MLMC_MAX_LEVELS + 1];
    uint64_t level_costs[KX_MLMC_MAX_LEVELS + 1];
    uint64_t level_paths[KX_MLMC_MAX_LEVELS + 1];
    uint64_t total_cost;
} kx_mlmc_result;

/* price_mlmc_detailed (src/mlmc.rs:107-215): the telescoping sum of level
 * means E[P_l - P_(l-1)] over uniform grids of 2^l steps on [0, horizon],
 * GBM or Heston (simulate_level_pair, simulator.rs:321-409 and 592-690: the
 * coarse path of a pair steps with the summed normals of two fine steps).
 * A pilot of pilot_paths per level, then optimal_allocation's extra paths
 * with the seed XOR 0xA5A55A5ADEADBEEF (mlmc.rs:142-166). Each phase is two
 * path launches (all levels' fine paths, then all coarse paths) and one
 * statistics launch of the per-path differences. Path i of level l draws the
 * Philox stream keyed by mix(mix(seed, l), l + 1) (mix: simulator.rs:431). */
kx_status kx_price_mlmc(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                        const kx_mlmc_cfg *mcfg, kx_mlmc_result *out);

/* estimate_variance_at_level (mlmc.rs:218-229): the sample variance of
 * P_l - P_(l-1) over n_pilot coupled paths of level `level`. */
kx_status kx_mlmc_level_variance(const kx_program *prog, const kx_model *model, const kx_mc_config *cfg,
                                 uint32_t level, uint64_t n_pilot, double *variance);

/* optimal_allocation (mlmc.rs:231-258): paths per level
 * ceil(sum_k sqrt(V_k C_k) sqrt(V_l / C_l) / target), at least 1; all zero when
 * n is 0 or target <= 0. Host arithmetic only. */
kx_status kx_mlmc_optimal_allocation(const double *variances, const uint64_t *costs, size_t n, double target_var,
                                     uint64_t *out);

/* Pathwise adjoint: one reverse sweep per path recomputing the path from its
 * Philox counters with a checkpoint every `checkpoint_every` steps; the
 * barrier indicator of until-conditions is a logistic of the stated width.
 * No reference counterpart (the reference only bumps). */
kx_status kx_greeks_adjoint(const kx_program *prog, const kx_model *model,
                            const kx_mc_config *cfg, const kx_adjoint_cfg *acfg,
                            kx_sens *out);

/* price_american_lsm (src/lsm.rs:80-124): Longstaff-Schwartz on the grid
 * [0, dates...] with the monomial basis {1, S, ..., S^(n_basis-1)}
 * (lsm.rs:259-288) and Gauss elimination with partial pivoting
 * (numerics.rs:190-236). Paths are stored in HBM (FP32 or FP64 per
 * cfg->precision), the Gram matrix is block-reduced in FP64. */
kx_status kx_price_american_lsm(const kx_program *prog, const kx_model *model,
                                const kx_mc_config *cfg, const double *dates,
                                size_t n_dates, int32_t n_basis,
                                kx_price_result *out);

/* kx_price_american_lsm with a choice of regression basis (the reference has
 * only the monomials): KX_LSM_MONOMIAL = kx_price_american_lsm;
 * KX_LSM_LAGUERRE regresses on the weighted Laguerre functions
 * e^(-x/2) L_j(x), j < n_basis, of x = S / s0 (s0 the model's spot). */
#define KX_LSM_MONOMIAL 0
#define KX_LSM_LAGUERRE 1
kx_status kx_price_american_lsm_basis(const kx_program *prog, const kx_model *model,
                                      const kx_mc_config *cfg, const double *dates,
                                      size_t n_dates, int32_t n_basis, int32_t basis,
                                      kx_price_result *out);

/* kx_price_american_lsm_basis with every path's discounted realised value
 * (lsm.rs:226) in per_path_pv (nullable, cfg->n_paths doubles): the value of
 * the payoff at the date the path is exercised, discounted to t = 0, so a
 * caller can compare exercise decisions path by path. */
kx_status kx_price_american_lsm_paths(const kx_program *prog, const kx_model *model,
                                      const kx_mc_config *cfg, const double *dates,
                                      size_t n_dates, int32_t n_basis, int32_t basis,
                                      kx_price_result *out, double *per_path_pv);

/* n independent kx_price_american_lsm_basis problems in one call (no
 * reference counterpart; the reference prices one American option per
 * call, lsm.rs:80-124). Case i is progs[i] under models[i] with cfgs[i] on
 * the dates dates[i][0 .. n_dates[i]); all cases share n_basis and basis,
 * draw from Philox and have one precision. The backward induction of every
 * case still active at a date runs in one launch, and different cases'
 * dates overlap; out[i] equals, bit for bit, the result of
 * kx_price_american_lsm_basis on case i alone. At most 1024 cases. */
kx_status kx_price_american_lsm_batch(size_t n, const kx_program *const *progs,
                                      const kx_model *models, const kx_mc_config *cfgs,
                                      const double *const *dates, const size_t *n_dates,
                                      int32_t n_basis, int32_t basis, kx_price_result *out);

/* ---- books: a portfolio priced by replaying one CUDA graph ------------------
 * No reference counterpart (the reference prices contract by contract,
 * pricer.rs:97, or one shared simulation, pricer.rs:250). A book lowers and
 * binds its contracts once, keeps their tables in device memory it owns,
 * groups them by (model kind, precision, kernel family) and captures the
 * pricing step (one persistent path kernel per group over its (contract,
 * path-block) work queue, the chunk statistics, the copy of the results) in
 * one CUDA graph. Each contract keeps its own model, n_paths, seed and
 * steps_per_year; prices equal kx_price's contract by contract. Philox only. */
typedef struct kx_book kx_book;
#define KX_BOOK_TUNE 1u /* time each group's register budgets and work-item
                           sizes on the book at creation, keep the fastest */
typedef struct kx_book_info {
    uint32_t n_contracts, n_groups;
    uint64_t n_paths, path_steps;  /* totals over the book */
    double tune_ms;                /* time spent tuning at creation */
    uint32_t group_kernel[4];      /* first 4 groups: 1 k_paths, 2 k_lean, 3 static, 4 static + average */
    uint32_t group_minb[4];        /* tuned register budget */
    uint32_t group_item_paths[4];  /* tuned paths per work item */
    uint32_t group_contracts[4];
} kx_book_info;
kx_status kx_book_create(size_t n, const kx_program *const *progs,
                         const kx_model *models, const kx_mc_config *cfgs,
                         uint32_t flags, kx_book **out);
/* Replays the graph; out receives n results, contract order. */
kx_status kx_book_price(kx_book *book, kx_price_result *out);
/* New model parameters (same kinds) for every contract, uploaded in place:
 * the next kx_book_price prices the same paths under the new market. */
kx_status kx_book_set_models(kx_book *book, const kx_model *models);
kx_status kx_book_get_info(const kx_book *book, kx_book_info *info);
void kx_book_free(kx_book *book);

/* Calibration microbenchmark (no reference counterpart): measured throughput
 * of one GPU pipe on device 0, used as the roofline denominator of the path
 * kernels. what = 0: MUFU (lg2/ex2/sin/cos approximations, results/s);
 * 1: FP32 FMA (FMAs/s); 2: 32-bit integer multiply-high (IMAD.HI/s, the
 * Philox multiply); 3: FP32 GBM steps/s of the bare simulation loop (Philox
 * draw, Box-Muller, log-space update; no contract, no scheduling), the
 * ceiling of the path kernels; 4: the same for FP32 Heston steps/s (2 normals
 * and the full-truncation Euler step per step). */
kx_status kx_measure_peak(int32_t what, double *ops_per_s);

/* Counters of the last pricing call (see kx_launch_stats). */
kx_status kx_last_launch_stats(kx_launch_stats *out);

/* Device name, SM count and the compute capability of device 0. */
kx_status kx_device_info(char *name, size_t cap, int32_t *sm_count,
                         int32_t *cc_major, int32_t *cc_minor);

#ifdef __cplusplus
}
#endif
#endif /* KONTRACT_GPU_H */
