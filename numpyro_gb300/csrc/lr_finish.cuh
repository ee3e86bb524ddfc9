// lr_finish.cuh -- the last step of the logistic-regression potential for one point, by one warp.
//
// The row-tiled potential kernels (FP32 CUDA cores, tcgen05 tensor cores) leave per-row-group
// partial gradients part_g[row_group][point][64] and log-likelihoods part_ll[row_group][point].
// Here they are summed and the Normal(0, s) prior added (numpyro's potential_energy of
// examples/covtype.py:66-71: U = -sum_n log Bernoulli(y_n | l_n) - sum_d log Normal(b_d; 0, s)):
//   dU/db_d = sum_groups part_g + b_d / s^2
//   U       = sum_groups part_ll + sum_d (b_d^2 / (2 s^2) + lin_d b_d) + pe_const
// lin is the tensor-core path's linear term (X'^T 1 / 2, null on CUDA cores); pe_const =
// p (log(2 pi) / 2 + log s) and inv_var_f = 1 / s^2 are formed once on the host.  Shared by the
// finish kernel and the state-machine kernel that fuses it, so both give the same bits.
//
// The tensor-core path (lin non-null) differs in two ways:
//  * e_tanh: its GEMM2 summed tanh(l'/2) X' = 2 sigmoid(l') X' - X'^T 1, so the likelihood
//    gradient is half the partial sums plus lin, and the gradient of the nonlinear part
//    N(b) = sum_n [softplus(l'_n) - l'_n / 2] is nu = half the partial sums.
//  * split3 (per block of 128 chains): 0 when the launch took the coefficients as two bf16
//    terms b_hm = 2 (hi + mid) of b / 2, leaving out b_lo = 2 lo (|b_lo| <= 2^-16 |b|).  Its
//    log-likelihood is then N(b_hm) + lin . b, and the first-order term nu(b_hm) . b_lo is added
//    here; the remainder is at most (1/8) lambda_max(X^T X) |b_lo|^2, which the launch held
//    below 1e-3 (otherwise it took all three terms and split3 is 1).  The gradient is the one
//    at b_hm: a deterministic function of b, which the leapfrog integrator may use (it stays
//    volume-preserving and reversible; only the energies decide acceptance).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace gbn {

__device__ __forceinline__ void logreg_finish_warp(const float* __restrict__ Q, int c, int npts, int ld, int p,
                                                   int row_groups, const float* __restrict__ part_g,
                                                   const double* __restrict__ part_ll,
                                                   const double* __restrict__ lin, float inv_var_f, double pe_const,
                                                   double* __restrict__ PE, float* __restrict__ G, int lane,
                                                   const int32_t* __restrict__ split3 = nullptr, bool e_tanh = false) {
  const double inv_var = (double)inv_var_f;
  const bool first_order = split3 && lin && split3[c >> 7] == 0;
  double lp = 0.0;
  for (int d = lane; d < p; d += 32) {
    const float bf = Q[(size_t)c * ld + d];
    // the row groups' FP32 gradient partials are summed in FP32 (the gradient is FP32); the
    // potential's prior and linear terms stay FP64 (lin . b reaches ~1e5 on large data)
    // (loads issued 8 at a time ahead of the in-order sum: the same sum, without a serialised
    // memory latency per row group)
    float s = 0.0f;
    const float* pg = part_g + (size_t)c * 64 + d;
    const size_t rs = (size_t)npts * 64;
    int r = 0;
    for (; r + 8 <= row_groups; r += 8) {
      float t[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) t[k] = pg[(size_t)(r + k) * rs];
#pragma unroll
      for (int k = 0; k < 8; ++k) s += t[k];
    }
    for (; r < row_groups; ++r) s += pg[(size_t)r * rs];
    double nu = 0.0;  // gradient of the nonlinear part of the log-likelihood
    if (e_tanh && lin) {
      nu = 0.5 * (double)s;
      s = (float)(nu + lin[d]);
    } else if (lin) {
      nu = (double)s - lin[d];
    }
    G[(size_t)c * ld + d] = fmaf(bf, inv_var_f, s);
    const double b = (double)bf;
    lp += 0.5 * b * b * inv_var;
    if (lin) lp += lin[d] * b;
    if (first_order) {  // b_lo = 2 lo, lo the third bf16 term of b / 2 (the split's own arithmetic)
      const float h = 0.5f * bf;
      const float r1 = h - __bfloat162float(__float2bfloat16_rn(h));
      const float r2 = r1 - __bfloat162float(__float2bfloat16_rn(r1));
      lp += nu * (2.0 * (double)r2);
    }
  }
  double ll = 0.0;
  for (int r = lane; r < row_groups; r += 32) ll += part_ll[(size_t)r * npts + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lp += __shfl_xor_sync(0xffffffffu, lp, o);
    ll += __shfl_xor_sync(0xffffffffu, ll, o);
  }
  if (lane == 0) PE[c] = ll + lp + pe_const;
}

}  // namespace gbn
