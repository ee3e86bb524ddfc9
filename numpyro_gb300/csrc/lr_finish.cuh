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
#pragma once
#include <cstdint>

namespace gbn {

__device__ __forceinline__ void logreg_finish_warp(const float* __restrict__ Q, int c, int npts, int ld, int p,
                                                   int row_groups, const float* __restrict__ part_g,
                                                   const double* __restrict__ part_ll,
                                                   const double* __restrict__ lin, float inv_var_f, double pe_const,
                                                   double* __restrict__ PE, float* __restrict__ G, int lane) {
  const double inv_var = (double)inv_var_f;
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
    G[(size_t)c * ld + d] = fmaf(bf, inv_var_f, s);
    const double b = (double)bf;
    lp += 0.5 * b * b * inv_var;
    if (lin) lp += lin[d] * b;
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
