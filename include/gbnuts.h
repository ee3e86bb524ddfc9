/*
 * gbnuts.h -- C ABI of the GB300-native NUTS/HMC engine (libgbnuts.so).
 *
 * The library replaces the device arithmetic of numpyro's vectorized-chain
 * NUTS/HMC transition.  Each entry point below names the reference interface
 * it stands in for (paths relative to the numpyro source tree):
 *
 *   gbn_create / gbn_destroy      NUTS.__init__ / HMC.__init__        numpyro/infer/hmc.py:625-686, :916-951
 *                                 (model = registry family + data; potential_energy numpyro/infer/util.py:333-358)
 *   gbn_init                      HMC.init (vmapped hmc_init_fn)      numpyro/infer/hmc.py:740-799, init_kernel :193-362,
 *                                 find_valid_initial_params           numpyro/infer/util.py:366-508
 *   gbn_sample                    HMC.sample (vmapped sample_kernel)  numpyro/infer/hmc.py:806-816, :459-530
 *   gbn_run                       MCMC.run, chain_method="vectorized" numpyro/infer/mcmc.py:635-729 with fori_collect
 *                                 numpyro/util.py:321-454 (whole warmup+sampling loop on the device)
 *   gbn_potential_and_grad        value_and_grad(potential_fn)        numpyro/infer/hmc_util.py:242-252
 *   gbn_potential_vjp             jax.vjp of potential_fn (adjoint)   numpyro/infer/hmc_util.py:242-252
 *   gbn_last_error                RuntimeError text of init failure   numpyro/infer/util.py:800-832
 *
 * Conventions: every entry point is extern "C", returns an int status
 * (GBN_OK = 0), never throws, and never synchronises the caller's stream
 * except where documented (gbn_init and gbn_run poll a device counter).
 * Pointers named d_* are device pointers owned by the caller; the library
 * owns its model data and scratch inside the handle.  Handles are not
 * thread-safe; distinct handles are independent.
 */
#ifndef GBNUTS_H
#define GBNUTS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBN_ABI_VERSION 2

/* status codes */
#define GBN_OK 0
#define GBN_ERR_INVALID_ARG 1
#define GBN_ERR_SHAPE 2
#define GBN_ERR_CUDA 3
#define GBN_ERR_TIMEOUT 4      /* tick budget exhausted / device wait gave up */
#define GBN_ERR_INIT_FAILED 5  /* no finite potential after 100 init attempts */
#define GBN_ERR_UNSUPPORTED 6
#define GBN_ERR_OOM 7

/* model families (the potential registry) */
#define GBN_FAMILY_HIER_NC 1   /* non-centred hierarchical normal, many datasets  */
#define GBN_FAMILY_LOGREG 2    /* Bernoulli-logit GLM, Normal(0,1) prior          */
#define GBN_FAMILY_HORSESHOE 3 /* Gaussian GLM, horseshoe prior                   */
/* GBN_FAMILY_HORSESHOE hyper: [0] = 1 selects unscaled_betas ~ Normal(0, 1), beta = tau lambda
 * unscaled_betas (0: beta ~ Normal(0, tau lambda) sampled directly). */
#define GBN_FAMILY_SV 4        /* Gaussian random walk + StudentT volatility      */
/* GBN_FAMILY_SV hyper: [0] s rate (Exponential), [1] nu rate (Exponential), [2] = 1 selects the
 * non-centred walk h = s * cumsum(h_base), h_base ~ Normal(0, 1)^T (0: centred, as numpyro's
 * GaussianRandomWalk site). */

/* engines */
#define GBN_ENGINE_FUSED 0 /* per-chain trees, no lock-step, fused/tensor-core potentials */
#define GBN_ENGINE_PLAIN 1 /* lock-step masked trees (numpyro vmap semantics), FP32 CUDA-core potentials */
#define GBN_ENGINE_TICKS 2 /* per-chain trees on the launch-per-leapfrog tick engine (no persistent kernel) */
/* GBN_ENGINE_FUSED runs the hierarchical family (a warp per chain) and the stochastic-volatility
 * family (a CTA per chain) in one persistent launch that pulls chains from a device work queue;
 * other families use the tick engine. */

/* algorithms */
#define GBN_ALGO_NUTS 0
#define GBN_ALGO_HMC 1

/* potential precision (logistic family) */
#define GBN_PREC_FP32 0   /* FP32 CUDA cores */
#define GBN_PREC_BF16X3 1 /* tcgen05 BF16 split precision, FP32 accumulate */

typedef struct gbn_handle_s* gbn_handle;

/* Model description; host pointers, copied to the device by gbn_create. */
typedef struct {
  int32_t family;
  int32_t num_models; /* HIER_NC: number of independent datasets; else 1 */
  int64_t n;          /* rows (LOGREG/HORSESHOE), total groups (HIER_NC), T (SV) */
  int32_t p;          /* features (LOGREG/HORSESHOE); unused otherwise */
  const float* x;     /* [n][p] row-major design matrix (LOGREG, HORSESHOE) */
  const float* y;     /* [n] responses / observations / returns */
  const float* sigma; /* [n] observation sd (HIER_NC) */
  const int32_t* offsets; /* [num_models+1] group offsets (HIER_NC) */
  double hyper[8];    /* prior hyper-parameters, family specific (see models.py) */
} gbn_model_desc;

/* Kernel configuration: numpyro NUTS/HMC constructor arguments. */
typedef struct {
  int32_t num_chains;
  int32_t chains_per_model; /* HIER_NC: chain c runs dataset c / chains_per_model */
  int32_t algo;
  int32_t engine;
  int32_t precision;
  int32_t max_tree_depth_warmup; /* max_tree_depth (d1, d2) */
  int32_t max_tree_depth;
  int32_t adapt_step_size;
  int32_t adapt_mass_matrix;
  int32_t dense_mass; /* 1: full mass matrices ([C][D][D] in gbn_state), latent dim <= 1024, not SV */
  int32_t regularize_mass_matrix;
  int32_t find_heuristic_step_size;
  int32_t num_steps; /* HMC: fixed number of steps, 0 = from trajectory_length */
  double target_accept_prob;
  double trajectory_length; /* HMC */
  double max_delta_energy;  /* 1000 */
  double init_step_size;
  uint64_t seed;
  /* Block-structured mass matrices (numpyro's dense_mass as a list of site-name tuples,
   * hmc_util.py:439-486), with dense_mass = 1: NULL, or latent-dim entries, the dense block of
   * each coordinate (>= 0) or -1 for the coordinates the remaining diagonal block holds.  The
   * mass matrices stay [C][D][D] (block-diagonal); at each window end the Welford covariance keeps
   * only the entries within a block and the diagonal. */
  const int32_t* mass_blocks;
  /* Global id of the handle's chain 0 (>= 0).  Every random draw of chain c is addressed by
   * (seed, first_chain + c, iteration, purpose) in the counter-based Philox streams, so a run split
   * across handles or GPUs -- each with its own range of chains, one seed -- gives every chain the
   * draws it has in one handle of all the chains. */
  int32_t first_chain;
} gbn_config;

/* HMCState (numpyro/infer/hmc.py:31-47) + HMCAdaptState (hmc_util.py:18-30)
 * as caller-owned device buffers, chain-major.  C = num_chains, D = latent dim.
 * With dense_mass the three mass matrices are [C][D][D] row-major (inverse_mass_matrix
 * symmetric, mass_matrix_sqrt and mass_matrix_sqrt_inv lower triangular) and mm_m2 is
 * [C][D][D]; gbn_init's d_inverse_mass_matrix is then [C][D][D] as well. */
typedef struct {
  int32_t* i;                   /* [C] iteration */
  float* z;                     /* [C][D] unconstrained position */
  float* z_grad;                /* [C][D] */
  double* potential_energy;     /* [C] */
  double* energy;               /* [C] */
  int32_t* num_steps;           /* [C] leapfrog steps of the last trajectory */
  float* accept_prob;           /* [C] */
  float* mean_accept_prob;      /* [C] */
  uint8_t* diverging;           /* [C] */
  float* step_size;             /* [C] adapt_state.step_size */
  float* inverse_mass_matrix;   /* [C][D] diagonal ([C][D][D] dense) */
  float* mass_matrix_sqrt;      /* [C][D] ([C][D][D] dense) */
  float* mass_matrix_sqrt_inv;  /* [C][D] ([C][D][D] dense) */
  double* ss_state;             /* [C][5] dual averaging (x_t, x_avg, g_avg, t, prox_center) */
  double* mm_mean;              /* [C][D] Welford mean */
  double* mm_m2;                /* [C][D] Welford m2 ([C][D][D] dense) */
  int32_t* mm_n;                /* [C] */
  int32_t* window_idx;          /* [C] */
  uint32_t* rng_key;            /* [C][2] (chain id, transition counter) */
} gbn_state;

/* Per-iteration collection buffers for gbn_run (any pointer may be NULL). */
typedef struct {
  float* samples;          /* [C][S][D] z (unconstrained) */
  int32_t* num_steps;      /* [C][S] */
  float* accept_prob;      /* [C][S] */
  uint8_t* diverging;      /* [C][S] */
  double* potential_energy;/* [C][S] */
  float* step_size;        /* [C][S] */
} gbn_collect;

typedef struct {
  int64_t ticks;          /* device ticks (one leapfrog for every pending chain) */
  int64_t grad_evals;     /* gradient evaluations consumed by chains */
  int64_t potential_launches;
  double device_ms;       /* CUDA-event time of the last gbn_run/gbn_sample */
} gbn_stats;

int gbn_abi_version(void);
/* 1 when this GPU runs the tcgen05 (sm_103a) tensor-core potentials, else 0 */
int gbn_tc_available(void);
const char* gbn_last_error(gbn_handle h); /* h may be NULL: last global error */

int gbn_create(gbn_handle* out, const gbn_model_desc* model, const gbn_config* cfg);
int gbn_destroy(gbn_handle h);
/* Integer id of a handle (unique in the process, assigned by gbn_create; 0 for NULL) and the
 * handle of an id (NULL once destroyed), thread-safe: for callers that pass a handle as a plain
 * attribute, such as an XLA FFI handler bound through jax.ffi (numpyro's sample runs under jit,
 * numpyro/infer/mcmc.py:188-190), which XLA may invoke from any thread. */
int64_t gbn_handle_id(gbn_handle h);
gbn_handle gbn_handle_from_id(int64_t id);
int gbn_latent_dim(gbn_handle h, int32_t* dim);

/* U(z) and dU/dz for num_points latent vectors (device pointers). */
int gbn_potential_and_grad(gbn_handle h, void* stream, const float* d_z, int32_t num_points,
                           double* d_pe, float* d_grad);
/* Vector-Jacobian product of U: d_out = cot[k] * dU/dz(z_k).  Allocates nothing when
 * num_points <= num_chains (the handle's scratch is sized for that many points at gbn_create). */
int gbn_potential_vjp(gbn_handle h, void* stream, const float* d_z, int32_t num_points,
                      const double* d_cot, float* d_out);

/* Initialise every chain: init_to_uniform(radius=2) when d_init_z is NULL,
 * validity retries, initial adaptation state. */
int gbn_init(gbn_handle h, void* stream, int32_t num_warmup, const float* d_init_z,
             const float* d_inverse_mass_matrix, gbn_state* st);

/* One transition for every chain (MCMCKernel.sample). */
int gbn_sample(gbn_handle h, void* stream, gbn_state* st);

/* The same transition, enqueued on `stream` with no host synchronisation, for callers that
 * trace sample(): numpyro runs it under jit (numpyro/infer/mcmc.py:188-190, util.py:386-403),
 * where an XLA FFI handler must not block the host.  The tick engine's loop runs on the device:
 * a CUDA graph whose WHILE node repeats batches of ticks until no chain is active, bounded by a
 * tick budget; the hierarchical and stochastic-volatility families are one persistent launch.
 * The first call on a handle builds that graph (a synchronous set-up). Draws and states are
 * bit-identical to gbn_sample.  A budget exhausted or a device wait timed out is recorded on the
 * device and reported by gbn_check_async. */
int gbn_sample_async(gbn_handle h, void* stream, gbn_state* st);
/* Synchronises `stream` and returns GBN_ERR_TIMEOUT if an earlier gbn_sample_async ran out of
 * its tick budget or a tensor-core wait timed out (the error is then cleared), else GBN_OK. */
int gbn_check_async(gbn_handle h, void* stream);

/* num_iterations transitions per chain; iteration j (0-based, this call) is
 * collected when j >= collect_start and (j - collect_start) % thinning == 0. */
int gbn_run(gbn_handle h, void* stream, gbn_state* st, int32_t num_iterations,
            int32_t collect_start, int32_t thinning, gbn_collect* out);

int gbn_get_stats(gbn_handle h, gbn_stats* stats);
/* Launch shapes the autotuner chose at gbn_create for this model's potential kernels ("name=value ...",
 * empty when nothing was tuned).  The autotuner times the candidate chains-per-CTA / tile shapes
 * once per process for each (device, model shape, chain count); GBN_AUTOTUNE=0 in the environment
 * keeps the defaults.  No counterpart in the reference. */
const char* gbn_tuning(gbn_handle h);

/* Measurement utility, no counterpart in the reference: the mean CUDA-event time (ms) of `reps`
 * back-to-back launches of the handle's potential over all its chains, at their last query
 * positions, in the form the tick engine launches it (for the tensor-core logistic potential the
 * tcgen05 kernel alone: its coefficient split and finish run inside the state-machine kernel).
 * Call it between runs, not during one. */
int gbn_time_potential(gbn_handle h, void* stream, int32_t reps, float* ms);
/* Measurement utility, no counterpart in the reference: the peak throughput (operations per
 * second, whole GPU) of the special-function unit on the operations of the tensor-core logistic
 * epilogue -- mode 0 ex2.approx, 1 tanh.approx, 2 the epilogue's mix (per 16 logits 16 ex2,
 * 8 tanh, 1 rcp, 2 lg2) -- measured with independent dependency chains on every SM (a few ms).  The
 * roofline of that kernel's special-function work is taken against it. */
int gbn_measure_sfu(void* stream, int32_t mode, double* ops_per_second);

/* Diagnostic, no counterpart in the reference: for a tensor-core logistic handle, how many of the
 * 128-chain blocks of its last potential launch took all three bf16 terms of the coefficients
 * (the others took two and a first-order term, exact to 1e-3; logreg_tc.cu), of how many blocks,
 * and the bound on a block's largest sum of squares of the third terms below which it takes two
 * (negative: always three).  Other handles report 0 blocks.  Call between runs (it waits for the
 * device). */
int gbn_logreg_terms(gbn_handle h, int32_t* three_term_blocks, int32_t* blocks, float* two_term_limit);

/* Largest num_points accepted by gbn_logreg_potential_noalloc. */
#define GBN_NOALLOC_MAX_POINTS 256

/* Logistic-regression U(z) and dU/dz (FP32 CUDA cores, same arithmetic as the
 * LOGREG family) that allocates no device memory, for callers that cannot call
 * cudaMalloc: a JAX/XLA FFI handler (XLA owns the device buffers and must not see
 * allocations per call), hosts that manage all device memory in their own pool.
 * No counterpart in the reference.  d_x [n][p] row-major, d_y [n], d_z
 * [num_points][p], d_pe [num_points], d_grad [num_points][p]; requires
 * 1 <= num_points <= GBN_NOALLOC_MAX_POINTS, 1 <= p <= 64 and a finite
 * prior_scale > 0, else GBN_ERR_INVALID_ARG.  Its scratch is a static device
 * array of about 1 MB that every GPU loading the library holds until exit, shared
 * by all calls: calls that overlap on the GPU race and must be serialised by the
 * caller.  The first call on a device performs the set-up (symbol addresses, the
 * kernel's shared-memory limit) and should come before any stream capture. */
int gbn_logreg_potential_noalloc(void* stream, const float* d_x, const float* d_y, int64_t n, int32_t p,
                                 double prior_scale, const float* d_z, int32_t num_points, double* d_pe,
                                 float* d_grad);
const char* gbn_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GBNUTS_H */
