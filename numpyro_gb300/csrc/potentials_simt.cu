// potentials_simt.cu -- FP32 CUDA-core potentials and hand-written adjoints.
//
// Every kernel evaluates numpyro's potential_energy (numpyro/infer/util.py:333-358)
// for a batch of latent points (one per chain) and its gradient, written by
// hand (no autodiff).  Log-densities follow numpyro/distributions:
//   Normal continuous.py:2975-2989, Cauchy :390-406, HalfCauchy :1149-1150,
//   HalfNormal :1190-1191, Exponential :715-726, StudentT :3229-3238,
//   GaussianRandomWalk :1104-1112, BernoulliLogits discrete.py:263 with
//   binary_cross_entropy_with_logits distributions/util.py:317-320;
// positive sites use biject_to(positive) = ExpTransform with log|det J| = x
// (transforms.py:641-644, :2115-2118).  Per-term arithmetic is FP32, sums
// are accumulated in FP64 so potential differences stay exact to ~1e-9
// relative even for 581k-row likelihoods.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include <cmath>

#include "common.cuh"
#include "hier_potential.cuh"
#include "internal.h"
#include "hs_finish.cuh"
#include "lr_finish.cuh"
#include "sv_potential.cuh"

namespace gbn {

constexpr double LOG_2PI = 1.8378770664093453;
constexpr double LOG_PI = 1.1447298858494002;
constexpr double LOG_2 = 0.6931471805599453;

// ============================================================ hierarchical (non-centred)
// z = [mu, log tau, theta_base(J)];  warp per point; model m = point / cpm
__global__ void __launch_bounds__(512) hier_nc_kernel(const float* __restrict__ Q, int npts, int ld,
                                                      const float* __restrict__ y, const float* __restrict__ sinv,
                                                      const double* __restrict__ cmodel,
                                                      const int32_t* __restrict__ off, int cpm, int num_models,
                                                      float inv_ms2, float inv_ts, double* __restrict__ PE,
                                                      float* __restrict__ G, const int32_t* pending) {
  if (pending && *pending == 0) return;
  int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);  // a warp per point
  int lane = threadIdx.x & 31;
  if (c >= npts) return;
  int m = c / cpm;
  if (m >= num_models) m = num_models - 1;  // points beyond the configured chains reuse the last model
  int j0 = off[m], J = off[m + 1] - j0;
  hier_nc_potential_warp(Q + (size_t)c * ld, G + (size_t)c * ld, PE + c, J, y + j0, sinv + j0, cmodel[m], inv_ms2,
                         inv_ts, lane);
}

// ============================================================ logistic regression (FP32 SIMT)
// Fused per row tile: logits = X_tile B^T -> (sigmoid, softplus) -> grad += E^T X_tile.
constexpr int LR_RT = 64;  // rows per tile
constexpr int LR_CT = 64;  // chains per CTA

__global__ void __launch_bounds__(256) logreg_simt_kernel(const float* __restrict__ X, const float* __restrict__ y,
                                                          int64_t N, int p, int DP, const float* __restrict__ Q,
                                                          int npts, int ld, float* __restrict__ part_g,
                                                          double* __restrict__ part_ll, int row_groups,
                                                          const int32_t* pending) {
  if (pending && *pending == 0) return;
  extern __shared__ __align__(16) float smem[];
  float* XsT = smem;                // [DP][RT]
  float* Xs = XsT + DP * LR_RT;     // [RT][DP]
  float* BsT = Xs + LR_RT * DP;     // [DP][CT]
  float* Es = BsT + DP * LR_CT;     // [RT][CT]
  float* ys = Es + LR_RT * LR_CT;   // [RT]
  double* red = (double*)(ys + LR_RT);  // [16][CT]
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const int c0 = blockIdx.x * LR_CT;
  const int rg = blockIdx.y;
  // chain coefficients, transposed
  for (int k = tid; k < DP * LR_CT; k += 256) {
    int cc = k / DP, d = k % DP;
    float v = 0.0f;
    if (d < p && c0 + cc < npts) v = Q[(size_t)(c0 + cc) * ld + d];
    BsT[d * LR_CT + cc] = v;
  }
  const int cg = tid & 15, dg = tid >> 4;  // phase-3 mapping
  const bool g_active = dg * 4 < DP;
  float gacc[4][4];
  double llacc[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    llacc[i] = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) gacc[i][j] = 0.0f;
  }
  int64_t ntiles = (N + LR_RT - 1) / LR_RT;
  for (int64_t tile = rg; tile < ntiles; tile += row_groups) {
    int64_t r0 = tile * LR_RT;
    __syncthreads();
    for (int k = tid; k < LR_RT * DP; k += 256) {
      int r = k / DP, d = k % DP;
      float v = 0.0f;
      if (d < p && r0 + r < N) v = X[(r0 + r) * (int64_t)p + d];
      Xs[r * DP + d] = v;
      XsT[d * LR_RT + r] = v;
    }
    if (tid < LR_RT) ys[tid] = (r0 + tid < N) ? y[r0 + tid] : 0.0f;
    __syncthreads();
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    for (int d = 0; d < DP; ++d) {
      float4 xv = *reinterpret_cast<const float4*>(&XsT[d * LR_RT + ty * 4]);
      float4 bv = *reinterpret_cast<const float4*>(&BsT[d * LR_CT + tx * 4]);
      float xa[4] = {xv.x, xv.y, xv.z, xv.w};
      float ba[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(xa[i], ba[j], acc[i][j]);
    }
    float llt[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // this tile's 4 rows, folded into FP64 once per tile
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int r = ty * 4 + i;
      bool rv = (r0 + r) < N;
      float yy = ys[r];
      float ev[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float l = acc[i][j];
        float t = expf(-fabsf(l));
        float sp = fmaxf(l, 0.0f) + log1pf(t);
        float inv = 1.0f / (1.0f + t);
        float sig = (l >= 0.0f) ? inv : t * inv;
        bool v = rv && (c0 + tx * 4 + j) < npts;
        ev[j] = v ? (sig - yy) : 0.0f;
        llt[j] += v ? (sp - yy * l) : 0.0f;
      }
      *reinterpret_cast<float4*>(&Es[r * LR_CT + tx * 4]) = make_float4(ev[0], ev[1], ev[2], ev[3]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) llacc[j] += (double)llt[j];
    __syncthreads();
    if (g_active) {
      for (int r = 0; r < LR_RT; ++r) {
        float4 e4 = *reinterpret_cast<const float4*>(&Es[r * LR_CT + cg * 4]);
        float4 x4 = *reinterpret_cast<const float4*>(&Xs[r * DP + dg * 4]);
        float ea[4] = {e4.x, e4.y, e4.z, e4.w};
        float xa[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) gacc[i][j] = fmaf(ea[i], xa[j], gacc[i][j]);
      }
    }
  }
  // partial gradient [rg][chain][64]
  if (g_active) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      int cc = c0 + cg * 4 + i;
      if (cc < npts) {
        float* dst = part_g + ((size_t)rg * npts + cc) * 64 + dg * 4;
        *reinterpret_cast<float4*>(dst) = make_float4(gacc[i][0], gacc[i][1], gacc[i][2], gacc[i][3]);
      }
    }
  }
  // log-likelihood partials: reduce over ty
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 4; ++j) red[ty * LR_CT + tx * 4 + j] = llacc[j];
  __syncthreads();
  if (tid < LR_CT) {
    double s = 0.0;
    for (int k = 0; k < 16; ++k) s += red[k * LR_CT + tid];
    if (c0 + tid < npts) part_ll[(size_t)rg * npts + c0 + tid] = s;
  }
}

// sum partials, add the N(0, scale) prior; warp per point
// lin (optional, FP64 [p]): a linear term lin . b of the log-likelihood computed outside the kernel
__global__ void logreg_finish_kernel(const float* __restrict__ Q, int npts, int ld, int p, int row_groups,
                                     const float* __restrict__ part_g, const double* __restrict__ part_ll,
                                     const double* __restrict__ lin, float inv_var_f, double pe_const,
                                     double* __restrict__ PE, float* __restrict__ G, const int32_t* pending,
                                     const int32_t* __restrict__ split3 = nullptr, bool e_tanh = false) {
  if (pending && *pending == 0) return;
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= npts) return;
  logreg_finish_warp(Q, c, npts, ld, p, row_groups, part_g, part_ll, lin, inv_var_f, pe_const, PE, G,
                     threadIdx.x & 31, split3, e_tanh);
}

// 1 / s^2 (FP32, as the gradient uses it) and p (log(2 pi) / 2 + log s) of the Normal(0, s) prior
void logreg_prior_consts(double prior_scale, int p, float* inv_var_f, double* pe_const) {
  *inv_var_f = (float)(1.0 / (prior_scale * prior_scale));
  *pe_const = (double)p * (0.5 * LOG_2PI + std::log(prior_scale));
}

// ============================================================ horseshoe: FP32 GEMMs + prior terms
// Both contractions of the Gaussian GLM run as one "NN" SGEMM, C[m][n] = sum_k A[k][m] B[k][n],
// with A and B row-major and m/n contiguous (rows padded to a multiple of 4 floats, so every
// tile row is float4-aligned):
//   residuals  R[row][c]  = y[row] - sum_p Xt[p][row] Bt[p][c]       (Xt = X^T, Bt = beta^T)
//   adjoint    GB[c][p]   = sum_row R[row][c] X[row][p]              (split over row ranges)
// X^T and a padded X are built once per model; beta^T is packed from the chains' positions each
// tick.  64 x 64 tiles, 16-deep K steps double-buffered through registers; 4 x 4 outputs per
// thread.  Residual sums of squares per (row tile, chain) leave the GEMM in FP64.
constexpr int HS_BN = 64, HS_BK = 16;
constexpr int HS_MIN_BM = 32;     // smallest tile height offered to the tuner
constexpr int HS_MAX_SPLITS = 8;  // most row ranges offered to the tuner for the adjoint GEMM

// TM rows per thread: tiles of (16 TM) x 64 outputs, 256 threads.
template <int TM>
__global__ void __launch_bounds__(256) hs_sgemm_nn_kernel(const float* __restrict__ A, int lda,
                                                          const float* __restrict__ B, int ldb, int M, int N,
                                                          int K, int k_per_split, float* __restrict__ Out, int ldo,
                                                          int64_t split_stride, const float* __restrict__ yv,
                                                          double* __restrict__ part_rr, int ld_rr,
                                                          const int32_t* pending) {
  if (pending && *pending == 0) return;
  constexpr int BM = 16 * TM;
  constexpr int AQ = BM / 4;  // float4 per K row of the A tile
  __shared__ __align__(16) float As[2][HS_BK][BM];
  __shared__ __align__(16) float Bs[2][HS_BK][HS_BN];
  __shared__ float rr[16][HS_BN];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * HS_BN;
  const int kb = blockIdx.z * k_per_split, ke = min(K, kb + k_per_split);
  // per K step a thread stages one float4 of B (row lk, columns lc..lc+3) and, when tid < 4 BM,
  // one float4 of A (row ak, columns ac..ac+3)
  const int lk = tid >> 4, lc = (tid & 15) * 4;
  const bool a_loader = tid < HS_BK * AQ;
  const int ak = tid / AQ, ac = (tid % AQ) * 4;
  auto load = [&](int k0, float4& av, float4& bv) {
    const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
    av = (a_loader && k0 + ak < ke && m0 + ac < M)
             ? *reinterpret_cast<const float4*>(A + (size_t)(k0 + ak) * lda + m0 + ac)
             : zero;
    bv = (k0 + lk < ke && n0 + lc < N) ? *reinterpret_cast<const float4*>(B + (size_t)(k0 + lk) * ldb + n0 + lc)
                                       : zero;
  };
  float acc[TM][4] = {};
  float4 av, bv;
  load(kb, av, bv);
  int buf = 0;
  for (int k0 = kb; k0 < ke; k0 += HS_BK) {
    if (a_loader) *reinterpret_cast<float4*>(&As[buf][ak][ac]) = av;
    *reinterpret_cast<float4*>(&Bs[buf][lk][lc]) = bv;
    __syncthreads();
    if (k0 + HS_BK < ke) load(k0 + HS_BK, av, bv);  // next step's loads overlap this step's FMAs
#pragma unroll
    for (int kk = 0; kk < HS_BK; ++kk) {
      float aa[TM];
#pragma unroll
      for (int i = 0; i < TM; i += 2) {
        const float2 a2 = *reinterpret_cast<const float2*>(&As[buf][kk][ty * TM + i]);
        aa[i] = a2.x;
        aa[i + 1] = a2.y;
      }
      const float4 b4 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      const float bb[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(aa[i], bb[j], acc[i][j]);
    }
    buf ^= 1;  // the other buffer was last read before this step's barrier
  }
  float* out = Out + (size_t)blockIdx.z * split_stride;
  if (yv == nullptr) {
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int m = m0 + ty * TM + i;
      if (m >= M) continue;
      if (n0 + tx * 4 < N)
        *reinterpret_cast<float4*>(out + (size_t)m * ldo + n0 + tx * 4) =
            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    }
    return;
  }
  // residual epilogue: R = y - acc, and per-chain sums of R^2 over this row tile
  float sq[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty * TM + i;
    if (m >= M) continue;
    const float y = yv[m];
    float r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      r[j] = y - acc[i][j];
      sq[j] = fmaf(r[j], r[j], sq[j]);
    }
    if (n0 + tx * 4 < N) *reinterpret_cast<float4*>(out + (size_t)m * ldo + n0 + tx * 4) = make_float4(r[0], r[1], r[2], r[3]);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) rr[ty][tx * 4 + j] = sq[j];
  __syncthreads();
  if (tid < HS_BN && n0 + tid < N) {
    double t = 0.0;
    for (int k = 0; k < 16; ++k) t += (double)rr[k][tid];
    part_rr[(size_t)blockIdx.y * ld_rr + n0 + tid] = t;
  }
}

// Bt[p][c] = beta_c[p] (p < P, c < npts), zero in the padding; 32 x 32 tiles through shared memory.
// Centred: beta is z[0:P].  Non-centred: beta = exp(log tau + log lambda) * unscaled_beta.
__global__ void __launch_bounds__(256) hs_pack_kernel(const float* __restrict__ Q, int ld, int npts, int P,
                                                      int noncentred, float* __restrict__ Bt, int ldb, int prows,
                                                      const int32_t* pending) {
  if (pending && *pending == 0) return;
  __shared__ float t[32][33];
  const int c0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + k, p = p0 + tx;
    float v = 0.0f;
    if (c < npts && p < P) {
      const float* z = Q + (size_t)c * ld;
      v = noncentred ? expf(z[P + 1] + z[p]) * z[P + 2 + p] : z[p];
    }
    t[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int p = p0 + k, c = c0 + tx;
    if (p < prows && c < ldb) Bt[(size_t)p * ldb + c] = t[tx][k];
  }
}

// Prior terms and the gradient of the horseshoe GLM, one CTA per chain, FP32 per coordinate with
// float-float sums.  Centred: z = [beta(P), log lambda(P), log sigma, log tau] (sorted sites).
// Non-centred (unscaled_betas ~ Normal(0, 1), beta = tau lambda unscaled_beta, as
// examples/horseshoe_regression.py:33-49): z = [log lambda(P), log sigma, log tau, unscaled_beta(P)];
// with g = X^T R / sigma^2: dU/d unscaled_d = eta_d - tau lambda_d g_d, dU/d log lambda_d =
// -beta_d g_d + 2 lambda^2/(1+lambda^2) - 1, dU/d log tau = -sum_d beta_d g_d + 2 tau^2/(1+tau^2) - 1.
//   beta_d ~ Normal(0, tau lambda_d): 0.5 b^2/s^2 + log s, s = tau lambda  (the log lambda cancels
//   against the Exp log-det);  lambda_d, tau ~ HalfCauchy(1);  sigma ~ HalfNormal(1).
// log(1 + lambda^2) = 2 max(l, 0) + log1p(e^{-2|l|}) and 2 lambda^2/(1 + lambda^2) = 2 / (1 + e^{-2l})
// stay finite for any l.
__global__ void __launch_bounds__(256) horseshoe_finish_kernel(const float* __restrict__ Q, int npts, int ld, int P,
                                                               int64_t N, const float* __restrict__ part_gb,
                                                               int splits, int ldg, const double* __restrict__ part_rr,
                                                               int ld_rr, int mtiles, int noncentred,
                                                               double* __restrict__ PE, float* __restrict__ G,
                                                               const int32_t* pending) {
  if (pending && *pending == 0) return;
  __shared__ double red[16];
  horseshoe_finish_block(Q, blockIdx.x, ld, P, N, part_gb, splits, ldg, npts, part_rr, ld_rr, mtiles, noncentred, PE,
                         G, threadIdx.x, red);
}

// ============================================================ stochastic volatility
// z = [h(T) or h_base(T), log nu, log s]; CTA per point (sv_potential.cuh).
__global__ void __launch_bounds__(256) sv_kernel(const float* __restrict__ Q, int npts, int ld, int T,
                                                 const float* __restrict__ ret, double s_rate, double nu_rate,
                                                 int noncentred, double* __restrict__ PE, float* __restrict__ G,
                                                 const int32_t* pending) {
  if (pending && *pending == 0) return;
  __shared__ SvSmem<256> sm;
  const int c = blockIdx.x, tid = threadIdx.x;
  const float* z = Q + (size_t)c * ld;
  float* gz = G + (size_t)c * ld;
  if (noncentred)
    sv_nc_potential_block<256>(z, gz, PE + c, T, ret, s_rate, nu_rate, tid, sm);
  else
    sv_potential_block<256>(z, gz, PE + c, T, ret, s_rate, nu_rate, tid, sm);
}

__global__ void scale_rows_kernel(const double* __restrict__ cot, float* __restrict__ G, int npts, int D) {
  size_t total = (size_t)npts * D;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x)
    G[k] = (float)((double)G[k] * cot[k / D]);
}

// ============================================================ host side
static int logreg_dp(int p) { return ((p + 3) / 4) * 4; }

cudaError_t ensure_potential_scratch(ModelDev& m, int points) {
  if (points <= m.scratch_points) return cudaSuccess;
  free_potential_scratch(m);
  cudaError_t e = cudaSuccess;
  if (m.family == 2) {
    // row groups: enough CTAs for ~4 waves over 152 SMs; buffers hold twice that for the tuner
    int cgroups = (points + LR_CT - 1) / LR_CT;
    int64_t ntiles = (m.n + LR_RT - 1) / LR_RT;
    int rg = (int)((4 * 152 + cgroups - 1) / cgroups);
    if (rg < 1) rg = 1;
    if (rg > ntiles) rg = (int)ntiles;
    m.row_groups = rg;
    m.row_groups_cap = (int)std::min<int64_t>(2 * (int64_t)rg, ntiles);
    if (m.tune.lr_rg > m.row_groups_cap) m.tune.lr_rg = 0;
    e = cudaMalloc(&m.part_g, sizeof(float) * (size_t)m.row_groups_cap * points * 64);
    if (e == cudaSuccess) e = cudaMalloc(&m.part_ll, sizeof(double) * (size_t)m.row_groups_cap * points);
  } else if (m.family == 3) {
    const int cp = pad4(points), pp = pad4(m.p);
    const int mt = (int)((m.n + HS_MIN_BM - 1) / HS_MIN_BM);
    e = cudaMalloc(&m.resid, sizeof(float) * (size_t)m.n * cp);
    if (e == cudaSuccess) e = cudaMalloc(&m.part_rr, sizeof(double) * (size_t)mt * cp);
    if (e == cudaSuccess) e = cudaMalloc(&m.part_gb, sizeof(float) * (size_t)HS_MAX_SPLITS * points * pp);
    if (e == cudaSuccess) e = cudaMalloc(&m.hs_bt, sizeof(float) * (size_t)pp * cp);
  }
  if (e == cudaSuccess) {
    m.scratch_points = points;
    if (m.tc) e = logreg_tc_prepare(m, points);
  }
  return e;
}

void free_potential_scratch(ModelDev& m) {
  cudaFree(m.part_g);
  cudaFree(m.part_ll);
  cudaFree(m.resid);
  cudaFree(m.part_rr);
  cudaFree(m.part_gb);
  cudaFree(m.hs_bt);
  m.hs_bt = nullptr;
  m.part_g = nullptr;
  m.part_ll = nullptr;
  m.resid = nullptr;
  m.part_rr = nullptr;
  m.part_gb = nullptr;
  m.scratch_points = 0;
}

static size_t logreg_smem(int DP) {
  return sizeof(float) * (size_t)(DP * LR_RT + LR_RT * DP + DP * LR_CT + LR_RT * LR_CT + LR_RT) +
         sizeof(double) * 16 * LR_CT;
}

namespace {
std::mutex g_simt_attr_mu;
std::vector<char> g_simt_attr_done;  // per device ordinal: the shared-memory limit is raised
}  // namespace

// logreg_simt_kernel needs about 74 KB of dynamic shared memory at 64 features, above the 48 KB
// default.  The limit is a per-device attribute of the kernel, so it is raised once for every
// device the kernel runs on (with that device current), under a mutex.
cudaError_t logreg_simt_smem_attr() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_simt_attr_mu);
  if ((int)g_simt_attr_done.size() <= dev) g_simt_attr_done.resize((size_t)dev + 1, 0);
  if (g_simt_attr_done[(size_t)dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(logreg_simt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)logreg_smem(64));
  if (e == cudaSuccess) g_simt_attr_done[(size_t)dev] = 1;
  return e;
}

cudaError_t launch_potential(ModelDev& m, const float* Q, int npts, double* PE, float* G, const int32_t* pending,
                             cudaStream_t st, bool fused_tick) {
  if (npts <= 0) return cudaSuccess;
  cudaError_t e = ensure_potential_scratch(m, npts);
  if (e != cudaSuccess) return e;
  const int ld = m.D;
  switch (m.family) {
    case 1:
    {
      const int cpb = m.tune.hier_cpb;
      hier_nc_kernel<<<(npts + cpb - 1) / cpb, 32 * cpb, 0, st>>>(
          Q, npts, ld, m.y, m.hier_sinv, m.hier_cmodel, m.offsets, m.chains_per_model, m.num_models,
          (float)(1.0 / (m.hyper[0] * m.hyper[0])), (float)(1.0 / m.hyper[1]), PE, G, pending);
    }
      break;
    case 2: {
      if (m.precision == 1 && m.tc) return logreg_tc_launch(m, Q, npts, PE, G, pending, st, fused_tick);
      int DP = logreg_dp(m.p);
      size_t sm = logreg_smem(DP);
      e = logreg_simt_smem_attr();
      if (e != cudaSuccess) return e;
      const int rg = m.tune.lr_rg > 0 ? m.tune.lr_rg : m.row_groups;
      dim3 grid((npts + LR_CT - 1) / LR_CT, rg);
      logreg_simt_kernel<<<grid, 256, sm, st>>>(m.x, m.y, m.n, m.p, DP, Q, npts, ld, m.part_g, m.part_ll, rg,
                                                pending);
      float ivf;
      double pec;
      logreg_prior_consts(m.hyper[0], m.p, &ivf, &pec);
      logreg_finish_kernel<<<(npts + 7) / 8, 256, 0, st>>>(Q, npts, ld, m.p, rg, m.part_g, m.part_ll, nullptr, ivf,
                                                           pec, PE, G, pending);
      break;
    }
    case 3: {
      if (m.precision == 1 && m.hs_tc) return horseshoe_tc_launch(m, Q, npts, PE, G, pending, st, fused_tick);
      const int P = m.p, M = (int)m.n, cp = pad4(npts), pp = pad4(P);
      const int tm = m.tune.hs_tm, splits = m.tune.hs_splits, bm = 16 * tm;
      const int mt = (M + bm - 1) / bm;
      // beta^T for the chains' query points
      dim3 gp((cp + 31) / 32, (pp + 31) / 32);
      const int nc = m.hyper[0] != 0.0;
      hs_pack_kernel<<<gp, 256, 0, st>>>(Q, ld, npts, P, nc, m.hs_bt, cp, pp, pending);
      // R[row][c] = y[row] - sum_p X[row][p] beta_c[p]
      dim3 g1((npts + HS_BN - 1) / HS_BN, mt, 1);
      if (tm == 2)
        hs_sgemm_nn_kernel<2><<<g1, 256, 0, st>>>(m.hs_xt, pad4(M), m.hs_bt, cp, M, npts, P, P, m.resid, cp, 0,
                                                  m.y, m.part_rr, cp, pending);
      else
        hs_sgemm_nn_kernel<4><<<g1, 256, 0, st>>>(m.hs_xt, pad4(M), m.hs_bt, cp, M, npts, P, P, m.resid, cp, 0,
                                                  m.y, m.part_rr, cp, pending);
      // GB[s][c][p] = sum_{row in split s} R[row][c] X[row][p]
      const int kps = (((M + splits - 1) / splits) + HS_BK - 1) / HS_BK * HS_BK;
      dim3 g2((P + HS_BN - 1) / HS_BN, (npts + 63) / 64, splits);
      hs_sgemm_nn_kernel<4><<<g2, 256, 0, st>>>(m.resid, cp, m.hs_xp, pp, npts, P, M, kps, m.part_gb, pp,
                                                (int64_t)npts * pp, nullptr, nullptr, 0, pending);
      horseshoe_finish_kernel<<<npts, 256, 0, st>>>(Q, npts, ld, P, m.n, m.part_gb, splits, pp, m.part_rr, cp, mt,
                                                    nc, PE, G, pending);
      break;
    }
    case 4:
      sv_kernel<<<npts, 256, 0, st>>>(Q, npts, ld, (int)m.n, m.y, m.hyper[0], m.hyper[1], m.hyper[2] != 0.0, PE, G,
                                      pending);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ============================================================ autotuner
namespace {
std::mutex g_tune_mu;
std::map<std::string, TuneParams> g_tune_cache;

// mean CUDA-event time of one potential launch (after one untimed launch)
cudaError_t time_potential(ModelDev& m, const float* Q, int npts, double* PE, float* G, cudaStream_t st, int reps,
                           float* ms) {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = launch_potential(m, Q, npts, PE, G, nullptr, st);
  if (e == cudaSuccess) e = cudaEventRecord(a, st);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch_potential(m, Q, npts, PE, G, nullptr, st);
  if (e == cudaSuccess) e = cudaEventRecord(b, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float t = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  *ms = t / (float)reps;
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  return e;
}

std::string tune_report(const ModelDev& m) {
  char buf[160];
  switch (m.family) {
    case 1: snprintf(buf, sizeof(buf), "hier_chains_per_cta=%d", m.tune.hier_cpb); break;
    case 2:
      snprintf(buf, sizeof(buf), "logreg_row_groups=%d", m.tune.lr_rg > 0 ? m.tune.lr_rg : m.row_groups);
      break;
    case 3:
      snprintf(buf, sizeof(buf), "horseshoe_tile_rows=%d horseshoe_splits=%d", 16 * m.tune.hs_tm,
               m.tune.hs_splits);
      break;
    default: buf[0] = 0; break;
  }
  return std::string(buf);
}
}  // namespace

cudaError_t autotune_potential(ModelDev& m, const float* Q, int npts, double* PE, float* G, cudaStream_t st,
                               std::string* report) {
  int dev = 0;
  cudaGetDevice(&dev);
  char key[192];
  snprintf(key, sizeof(key), "%d|%d|%lld|%d|%d|%d|%d|%d|%g", dev, m.family, (long long)m.n, m.p, m.D, m.num_models,
           npts, m.precision, m.hyper[0]);
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tune_cache.find(key);
  cudaError_t e = ensure_potential_scratch(m, npts);
  if (e != cudaSuccess) return e;
  const char* forced = getenv("GBN_TUNE");  // "hier_cpb=16 hs_tm=2 hs_splits=8 lr_rg=32": fixed shapes
  if (forced && forced[0]) {
    int v = 0;
    const char* p;
    if ((p = strstr(forced, "hier_cpb=")) && sscanf(p + 9, "%d", &v) == 1 && (v == 4 || v == 8 || v == 16))
      m.tune.hier_cpb = v;
    if ((p = strstr(forced, "hs_tm=")) && sscanf(p + 6, "%d", &v) == 1 && (v == 2 || v == 4)) m.tune.hs_tm = v;
    if ((p = strstr(forced, "hs_splits=")) && sscanf(p + 10, "%d", &v) == 1 && v >= 1 && v <= HS_MAX_SPLITS)
      m.tune.hs_splits = v;
    if ((p = strstr(forced, "lr_rg=")) && sscanf(p + 6, "%d", &v) == 1 && v >= 1 && v <= m.row_groups_cap)
      m.tune.lr_rg = v;
  } else if (it != g_tune_cache.end()) {
    m.tune = it->second;
  } else {
    std::vector<TuneParams> cand;
    TuneParams t = m.tune;
    if (m.family == 1) {
      for (int cpb : {4, 8, 16}) {
        t.hier_cpb = cpb;
        cand.push_back(t);
      }
    } else if (m.family == 2 && !(m.precision == 1 && m.tc)) {
      for (int rg : {std::max(1, m.row_groups / 2), m.row_groups, m.row_groups_cap}) {
        t.lr_rg = rg;
        cand.push_back(t);
      }
    } else if (m.family == 3) {
      for (int tm : {2, 4})
        for (int sp : {2, 4, 8}) {
          t.hs_tm = tm;
          t.hs_splits = sp;
          cand.push_back(t);
        }
    }
    float best = 1e30f;
    TuneParams pick = m.tune;
    for (const TuneParams& c : cand) {
      m.tune = c;
      float ms = 0.0f;
      e = time_potential(m, Q, npts, PE, G, st, 3, &ms);
      if (e != cudaSuccess) return e;
      if (ms < best) {
        best = ms;
        pick = c;
      }
    }
    m.tune = pick;
    g_tune_cache[key] = pick;
  }
  if (report) *report = tune_report(m);
  return cudaSuccess;
}

// ============================================================ special-function throughput
// Peak rate of the special-function unit for the operations of the tensor-core logistic epilogue
// (ex2.approx, tanh.approx, rcp.approx, lg2.approx), measured with independent dependency chains
// (8 per thread) so the unit, not latency, sets the rate.  MIX issues them in the epilogue's
// proportion: per 16 logits 16 ex2, 8 tanh, 1 rcp and 2 lg2 (1.6875 per logit).
template <int MODE>
__global__ void __launch_bounds__(256) sfu_rate_kernel(int iters, float* __restrict__ out) {
  float v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = 0.25f + 0.01f * (float)(k + (threadIdx.x & 7));
  for (int i = 0; i < iters; ++i) {
    if (MODE == 2) {
#pragma unroll
      for (int k = 0; k < 16; ++k) asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(v[k & 7]) : "f"(-v[k & 7]));
#pragma unroll
      for (int k = 0; k < 8; ++k) asm volatile("tanh.approx.f32 %0, %1;" : "=f"(v[k]) : "f"(v[k]));
      asm volatile("rcp.approx.ftz.f32 %0, %1;" : "=f"(v[0]) : "f"(1.0f + v[0]));
      asm volatile("lg2.approx.ftz.f32 %0, %1;" : "=f"(v[1]) : "f"(1.5f + v[1]));
      asm volatile("lg2.approx.ftz.f32 %0, %1;" : "=f"(v[2]) : "f"(1.5f + v[2]));
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (MODE == 0)
          asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(v[k]) : "f"(-v[k]));
        else
          asm volatile("tanh.approx.f32 %0, %1;" : "=f"(v[k]) : "f"(v[k]));
      }
    }
  }
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += v[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = acc;  // every chain's result is stored
}

cudaError_t measure_sfu_rate(int mode, cudaStream_t st, double* ops_per_s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t a = nullptr, b = nullptr;
  float* out = nullptr;  // one float per thread: the chains' results, so none is dead code
  e = cudaMalloc(&out, sizeof(float) * (size_t)blocks * threads);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  auto launch = [&]() {
    if (mode == 0) sfu_rate_kernel<0><<<blocks, threads, 0, st>>>(iters, out);
    else if (mode == 1) sfu_rate_kernel<1><<<blocks, threads, 0, st>>>(iters, out);
    else sfu_rate_kernel<2><<<blocks, threads, 0, st>>>(iters, out);
  };
  if (e == cudaSuccess) {
    launch();  // warm-up
    e = cudaEventRecord(a, st);
  }
  const int reps = 5;
  for (int r = 0; r < reps && e == cudaSuccess; ++r) launch();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventRecord(b, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  float ms = 0.0f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  // operations per launch: per thread and iteration 8 (one per chain), or the mix's 27
  const double per_thread = (mode == 2 ? 27.0 : 8.0) * iters;
  if (e == cudaSuccess) *ops_per_s = per_thread * blocks * threads * reps / (ms * 1e-3);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (out) cudaFree(out);
  return e;
}

cudaError_t launch_scale_rows(const double* cot, float* G, int npts, int D, cudaStream_t st) {
  size_t total = (size_t)npts * D;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  if (blocks < 1) blocks = 1;
  scale_rows_kernel<<<blocks, 256, 0, st>>>(cot, G, npts, D);
  return cudaGetLastError();
}

}  // namespace gbn

namespace gbn {
// FP32 logistic potential with scratch supplied by the caller (no allocation):
// part_g needs row_groups * npts * 64 floats, part_ll row_groups * npts doubles.
cudaError_t launch_logreg_simt_scratch(const float* x, const float* y, int64_t n, int p, double prior_scale,
                                       const float* Q, int npts, int row_groups, float* part_g, double* part_ll,
                                       double* PE, float* G, cudaStream_t st) {
  cudaError_t e = logreg_simt_smem_attr();
  if (e != cudaSuccess) return e;
  int DP = logreg_dp(p);
  dim3 grid((npts + LR_CT - 1) / LR_CT, row_groups);
  logreg_simt_kernel<<<grid, 256, logreg_smem(DP), st>>>(x, y, n, p, DP, Q, npts, p, part_g, part_ll, row_groups,
                                                         nullptr);
  e = cudaGetLastError();  // checked per launch, so the first failing launch is the one reported
  if (e != cudaSuccess) return e;
  float ivf;
  double pec;
  logreg_prior_consts(prior_scale, p, &ivf, &pec);
  logreg_finish_kernel<<<(npts + 7) / 8, 256, 0, st>>>(Q, npts, p, p, row_groups, part_g, part_ll, nullptr, ivf, pec,
                                                       PE, G, nullptr);
  return cudaGetLastError();
}

void horseshoe_finish_launch(const float* Q, int npts, int ld, int P, int64_t N, const float* part_gb, int splits,
                             int ldg, const double* part_rr, int ld_rr, int mtiles, int noncentred, double* PE,
                             float* G, const int32_t* pending, cudaStream_t st) {
  horseshoe_finish_kernel<<<npts, 256, 0, st>>>(Q, npts, ld, P, N, part_gb, splits, ldg, part_rr, ld_rr, mtiles,
                                                noncentred, PE, G, pending);
}

void logreg_finish_launch(const float* Q, int npts, int ld, int p, int row_groups, const float* part_g,
                          const double* part_ll, const double* lin, double prior_scale, double* PE, float* G,
                          const int32_t* pending, cudaStream_t st, const int32_t* split3, bool e_tanh) {
  float ivf;
  double pec;
  logreg_prior_consts(prior_scale, p, &ivf, &pec);
  logreg_finish_kernel<<<(npts + 7) / 8, 256, 0, st>>>(Q, npts, ld, p, row_groups, part_g, part_ll, lin, ivf, pec, PE,
                                                       G, pending, split3, e_tanh);
}
}  // namespace gbn
