// common.cuh -- device-side building blocks shared by every kernel of libgbnuts.
//
//  * Philox4x32-10 (Salmon et al., SC'11) and the stream address layout
//    (chain, transition, purpose<<24 | idx, sub); identical to the oracle's.
//  * the per-chain NUTS control block (ChainCtl) and engine buffer tables.
//  * group reductions: a "group" is the set of threads that owns one chain
//    (a warp, or a whole CTA for large latent dimension).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <math.h>

namespace gbn {

// ---------------------------------------------------------------- Philox
enum Purpose : uint32_t {
  P_MOMENTUM = 0,
  P_DOUBLING = 1,
  P_LEAF = 2,
  P_INIT = 3,
  P_HMC_ACCEPT = 4,
  P_HEURISTIC = 5,
};
constexpr uint32_t INIT_TRANSITION = 0xFFFFFFFFu;

__host__ __device__ __forceinline__ void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c.x, hi0, lo0);
    mulhilo32(0xCD9E8D57u, c.z, hi1, lo1);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

struct Seed {
  uint32_t lo, hi;
};

__device__ __forceinline__ uint4 draw(Seed s, uint32_t chain, uint32_t n, uint32_t purpose, uint32_t idx,
                                      uint32_t sub) {
  return philox4x32_10(make_uint4(chain, n, (purpose << 24) | idx, sub), s.lo, s.hi);
}

// (word >> 8) * 2^-24: exact in float32 and float64
__device__ __forceinline__ double u01d(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }
__device__ __forceinline__ float u01f(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

// Standard normal number d of the block sequence at (chain, n, purpose, sub):
// block k = d/4 gives two Box-Muller pairs (cos, sin, cos, sin).
__device__ __forceinline__ float normal_at(Seed s, uint32_t chain, uint32_t n, uint32_t purpose, int d,
                                           uint32_t sub) {
  uint4 w = draw(s, chain, n, purpose, (uint32_t)(d >> 2), sub);
  int j = d & 3;
  uint32_t a = (j < 2) ? w.x : w.z;
  uint32_t b = (j < 2) ? w.y : w.w;
  float u0 = u01f(a), u1 = u01f(b);
  float rad = sqrtf(-2.0f * log1pf(-u0));
  float sn, cs;
  sincospif(2.0f * u1, &sn, &cs);
  return (j & 1) ? rad * sn : rad * cs;
}

__device__ __forceinline__ float uniform_at(Seed s, uint32_t chain, uint32_t n, uint32_t purpose, int d,
                                            uint32_t sub) {
  uint4 w = draw(s, chain, n, purpose, (uint32_t)(d >> 2), sub);
  int j = d & 3;
  uint32_t x = j == 0 ? w.x : (j == 1 ? w.y : (j == 2 ? w.z : w.w));
  return u01f(x);
}

// ---------------------------------------------------------------- math
__device__ __forceinline__ double logaddexp_d(double a, double b) {
  double m = fmax(a, b);
  if (m == -INFINITY) return -INFINITY;
  return m + log1p(exp(-fabs(a - b)));
}
__device__ __forceinline__ double sigmoid_d(double x) { return 1.0 / (1.0 + exp(-x)); }

// Tree weights and energy differences are carried in FP64; the transcendental factors applied
// to an FP64 difference are evaluated in FP32 (GB300 issues FP64 at a small fraction of the FP32
// rate and these run on every leaf of every chain).
// log(e^a + e^b): FP64 maximum plus an FP32 correction log1p(e^-|a-b|) (absolute error < 1e-7).
__device__ __forceinline__ double logaddexp_mixed(double a, double b) {
  double m = fmax(a, b);
  if (m == -INFINITY) return -INFINITY;
  return m + (double)log1pf(expf(-(float)fabs(a - b)));
}
// min(1, e^x) and 1 / (1 + e^-x) of an FP64 argument, in FP32
__device__ __forceinline__ float exp_min1_f(double x) { return fminf(expf((float)x), 1.0f); }
__device__ __forceinline__ float sigmoid_f(double x) { return 1.0f / (1.0f + expf(-(float)x)); }

// ---------------------------------------------------------------- float-float sums
// An unevaluated pair hi + lo of FP32 numbers (Dekker 1971).  ff_add is Knuth's exact two-sum
// of the leading parts plus the trailing parts, renormalised; it is commutative bit for bit, so a
// butterfly reduction leaves every lane with the same pair.  Group sums use it instead of FP64
// adds: about 2^-44 relative error, no FP64 instruction.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bp = s - a.hi;
  float e = (a.hi - (s - bp)) + (b.hi - bp);
  e += a.lo + b.lo;
  const float hi = s + e;
  return FF{hi, e - (hi - s)};
}
__device__ __forceinline__ FF ff_from(float x) { return FF{x, 0.0f}; }
__device__ __forceinline__ double ff_value(FF a) { return (double)a.hi + (double)a.lo; }
// hi + lo <= 0, decided exactly in FP32 (a renormalised pair has |lo| <= ulp(hi) / 2)
__device__ __forceinline__ bool ff_le0(FF a) { return a.hi < 0.0f || (a.hi == 0.0f && a.lo <= 0.0f); }
__device__ __forceinline__ FF ff_shfl_xor(FF v, int o) {
  return FF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// digamma by upward recurrence to x >= 6 and the asymptotic series
// psi(x) ~ ln x - 1/(2x) - sum_k B_2k / (2k x^2k) (Abramowitz & Stegun 6.3.18).
__host__ __device__ inline double digamma_d(double x) {
  double acc = 0.0;
  while (x < 6.0) {
    acc -= 1.0 / x;
    x += 1.0;
  }
  double r = 1.0 / x, r2 = r * r;
  double series = r2 * (1.0 / 12 - r2 * (1.0 / 120 - r2 * (1.0 / 252 - r2 * (1.0 / 240 - r2 * (1.0 / 132)))));
  return acc + log(x) - 0.5 * r - series;
}

// Compensated FP32 accumulator (two-sum; the error term is carried separately).
struct Comp32 {
  float s, c;
  __device__ __forceinline__ void add(float x) {
    float t = s + x;
    float bp = t - s;
    c += (s - (t - bp)) + (x - bp);
    s = t;
  }
  __device__ __forceinline__ float value() const { return s + c; }
};

// Long per-thread sums are accumulated in compensated FP32 and the shares summed across the
// group as float-float pairs, converted to FP64 for the scalar terms.
__device__ __forceinline__ double comp_total(const Comp32& a) { return (double)a.s + (double)a.c; }
__device__ __forceinline__ FF comp_ff(const Comp32& a) {  // renormalised pair (|c| << |s|)
  const float hi = a.s + a.c;
  return FF{hi, a.c - (hi - a.s)};
}

// FP32 digamma by the same recurrence and asymptotic series (A&S 6.3.18)
__device__ __forceinline__ float digamma_f(float x) {
  float acc = 0.0f;
  while (x < 6.0f) {
    acc -= 1.0f / x;
    x += 1.0f;
  }
  const float r = 1.0f / x, r2 = r * r;
  const float series =
      r2 * (1.0f / 12 - r2 * (1.0f / 120 - r2 * (1.0f / 252 - r2 * (1.0f / 240 - r2 * (1.0f / 132)))));
  return acc + logf(x) - 0.5f * r - series;
}

// ---------------------------------------------------------------- engine
enum Phase : int32_t {
  PH_IDLE = 0,
  PH_START = 1,   // begin a transition at the next advance
  PH_LEAF = 2,    // NUTS leaf gradient pending
  PH_WAIT = 3,    // lock-step barrier (plain engine)
  PH_DONE = 4,    // all transitions of this call done
  PH_HMC = 5,     // fixed-length HMC leapfrog pending
  PH_HEUR = 6,    // find_reasonable_step_size trial pending
  PH_HEUR_START = 7,
};
enum HeurCtx : int32_t { HC_INIT = 0, HC_WINDOW = 1 };

// Per-chain control block (128 bytes, one per chain, library-owned).
struct __align__(16) ChainCtl {
  int32_t phase;
  int32_t iters_left;     // transitions still to run in this call
  int32_t iters_done;     // transitions finished in this call
  int32_t depth;          // current tree depth (before the running doubling)
  int32_t dir;            // 1 = right
  int32_t max_depth_cur;
  int32_t tree_turning, tree_div;
  int32_t num_prop;       // tree num_proposals
  int32_t sub_num, sub_div, sub_turning;
  int32_t hmc_left, hmc_total;   // fixed-length HMC: steps left / total
  int32_t heur_trial, heur_dir, heur_last, heur_ctx;
  float step;             // step size of this transition (magnitude)
  float pad0;
  double energy0;         // H at the start of the transition
  double tree_w, tree_acc, pe_p, energy_p;
  double sub_w, sub_acc, pe_sp, energy_sp;
  double heur_step, heur_e0;
};

// Tree/integrator scratch, chain-major [C][D] (checkpoints [C][maxd][D]).
struct EngineBufs {
  float *z_l, *r_l, *g_l, *z_r, *r_r, *g_r;
  float *z_p, *g_p, *z_sp, *g_sp;
  float *rsum, *rsum_sub;
  float *r_ck, *rs_ck;
  float* Q;      // query positions handed to the potential
  float* G;      // gradients returned by the potential
  double* PE;    // potentials returned by the potential
  ChainCtl* ctl;
  int32_t* chain_dim;  // [C] per-chain latent dim (uneven models) or nullptr
  float* tmp;          // dense mass matrix: [C][D] vector scratch (nullptr otherwise)
  double* tmpd;        // dense mass matrix: [C][2][D] Welford deltas (nullptr otherwise)
};

struct StateBufs {  // mirrors gbn_state (mass matrices and mm_m2 are [C][D][D] when dense)
  int32_t* i;
  float* z;
  float* z_grad;
  double* potential_energy;
  double* energy;
  int32_t* num_steps;
  float* accept_prob;
  float* mean_accept_prob;
  uint8_t* diverging;
  float* step_size;
  float* inverse_mass_matrix;
  float* mass_matrix_sqrt;
  float* mass_matrix_sqrt_inv;
  double* ss_state;
  double* mm_mean;
  double* mm_m2;
  int32_t* mm_n;
  int32_t* window_idx;
  uint32_t* rng_key;
};

struct CollectBufs {  // mirrors gbn_collect
  float* samples;
  int32_t* num_steps;
  float* accept_prob;
  uint8_t* diverging;
  double* potential_energy;
  float* step_size;
};

// Everything the advance kernel needs; lives in device memory so captured
// CUDA graphs stay valid when the caller's buffers change between calls.
struct __align__(16) AdvParams {
  EngineBufs e;
  StateBufs s;
  CollectBufs col;
  const int32_t* window_end;
  int32_t num_windows;
  int32_t num_warmup;
  int32_t C, D, maxd;
  int32_t mtd_warmup, mtd;
  int32_t algo;
  int32_t adapt_step, adapt_mass, regularize, heuristic;
  int32_t lockstep;
  int32_t dense;  // mass matrices [C][D][D] (dense_mass=True) instead of [C][D]
  const int32_t* mass_block;  // [D] dense block of each coordinate, -1 diagonal; null: one dense block
  int32_t fixed_steps;
  int32_t collect_start, thinning, num_collect;
  float target_accept;
  double max_dE;
  double traj_len;
  Seed seed;
  int32_t* counters;    // [4]: (pending, active) for parity 0 and 1
  int32_t* done_count;  // lock-step barrier counts, [max iterations + 1]
  int32_t* error_word;  // device error status
  // The tensor-core logistic potential fused into the tick engine (lrf_part_g null: not fused):
  // the advance kernel finishes the previous tick's potential from its row-group partials
  // (logreg_finish_warp) and writes the bf16x3 coefficient splits of every position it queries.
  const float* lrf_part_g;
  const double* lrf_part_ll;
  const double* lrf_lin;
  uint16_t* lrf_bsplit;  // [chains, padded][3][64] bfloat16 bits
  double lrf_pe_const;
  float lrf_inv_var;
  int32_t lrf_row_groups;
  const int32_t* lrf_split3;  // per 128-chain block: 1 if the launch took three coefficient terms
  int32_t lrf_e_tanh;         // GEMM2 summed tanh(l'/2) X' (see lr_finish.cuh)
  // The tensor-core horseshoe potential fused into the tick engine's CTA-per-chain state machine
  // (hsf_part_gb null: not fused): it finishes the previous tick's potential for the chains that
  // queried it (hs_finish.cuh) and writes the bf16 hi/mid/lo terms of the coefficients of every
  // position it queries (what split_beta_kernel does).
  const float* hsf_part_gb;
  const double* hsf_part_rr;
  uint16_t* hsf_bs;  // [3][hsf_total] bfloat16 bits: point c, feature k at c * hsf_kp + k
  int64_t hsf_N;
  int64_t hsf_total;
  int32_t hsf_P, hsf_kp, hsf_splits, hsf_ldg, hsf_ld_rr, hsf_mtiles, hsf_nc, hsf_pad;
};

// ---------------------------------------------------------------- groups
template <int NT>
struct Group;

template <>
struct Group<32> {  // one warp per chain
  int tid;
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ FF sumff(FF v, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
    return v;
  }
  __device__ __forceinline__ void sum2ff(FF& a, FF& b, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = ff_add(a, ff_shfl_xor(a, o));
      b = ff_add(b, ff_shfl_xor(b, o));
    }
  }
  __device__ __forceinline__ double sum(double v, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
  __device__ __forceinline__ float sumf(float v, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
  }
  __device__ __forceinline__ double2 sum2(double2 v, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
  }
};

template <>
struct Group<256> {  // one CTA of 256 threads per chain; red must hold 16 doubles
  int tid;
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  // warp butterflies, then every thread folds the 8 warp pairs in the same order
  __device__ __forceinline__ FF sumff(FF v, double* red) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
    float2* r = reinterpret_cast<float2*>(red);
    __syncthreads();
    if ((tid & 31) == 0) r[tid >> 5] = make_float2(v.hi, v.lo);
    __syncthreads();
    FF t{r[0].x, r[0].y};
#pragma unroll
    for (int w = 1; w < 8; ++w) t = ff_add(t, FF{r[w].x, r[w].y});
    return t;
  }
  __device__ __forceinline__ void sum2ff(FF& a, FF& b, double* red) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a = ff_add(a, ff_shfl_xor(a, o));
      b = ff_add(b, ff_shfl_xor(b, o));
    }
    float2* r = reinterpret_cast<float2*>(red);
    __syncthreads();
    if ((tid & 31) == 0) {
      r[tid >> 5] = make_float2(a.hi, a.lo);
      r[8 + (tid >> 5)] = make_float2(b.hi, b.lo);
    }
    __syncthreads();
    FF ta{r[0].x, r[0].y}, tb{r[8].x, r[8].y};
#pragma unroll
    for (int w = 1; w < 8; ++w) {
      ta = ff_add(ta, FF{r[w].x, r[w].y});
      tb = ff_add(tb, FF{r[8 + w].x, r[8 + w].y});
    }
    a = ta;
    b = tb;
  }
  __device__ __forceinline__ double sum(double v, double* red) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += red[w];
    return t;
  }
  __device__ __forceinline__ float sumf(float v, double* red) const { return (float)sum((double)v, red); }
  __device__ __forceinline__ double2 sum2(double2 v, double* red) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    __syncthreads();
    if ((tid & 31) == 0) {
      red[tid >> 5] = v.x;
      red[8 + (tid >> 5)] = v.y;
    }
    __syncthreads();
    double2 t = make_double2(0.0, 0.0);
#pragma unroll
    for (int w = 0; w < 8; ++w) {
      t.x += red[w];
      t.y += red[8 + w];
    }
    return t;
  }
};

}  // namespace gbn
