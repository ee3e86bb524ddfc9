// hier_potential.cuh -- warp-level potential + adjoint of the non-centred
// hierarchical normal model, shared by the tick-engine kernel
// (potentials_simt.cu) and the persistent engine (nuts_engine.cu) so both
// produce bit-identical gradients.  z and g carry no __restrict__: the persistent
// engine writes z in the same launch, so its loads must not take the read-only path.
//
//   mu ~ Normal(0, mu_scale); tau ~ HalfCauchy(tau_scale) (Exp transform, log-det = log tau);
//   theta_base_j ~ Normal(0, 1); theta_j = mu + tau * theta_base_j  (numpyro/infer/reparam.py:154-191)
//   y_j ~ Normal(theta_j, sigma_j)
// Log-densities: Normal numpyro/distributions/continuous.py:2975-2989, HalfCauchy :1149-1150,
// Cauchy :390-406; Exp log-det transforms.py:641-644.  z = [mu, log tau, theta_base(J)].
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"

namespace gbn {

// Per-model data of the hierarchical family: for each group y_j and 1/sigma_j; for each model the
// constant  sum_j log sigma_j + (J + 1/2) log 2pi + log mu_scale + log tau_scale + log pi - log 2
// (the normalisers of the two Normal terms per group, the Normal(mu) and HalfCauchy(tau) priors),
// computed once on the host; and the reciprocal scales of the priors.
struct HierData {
  const float* y;
  const float* sinv;
  const double* cmodel;
  float inv_ms2;  // 1 / mu_scale^2
  float inv_ts;   // 1 / tau_scale
};

// Potential and gradient of one model's chain, a warp per chain.  Per group everything is FP32
// multiplies (no division or logarithm), summed across the warp as float-float pairs; the
// scalar prior terms use FP32 exp/log1p, and only the final sum is FP64.
__device__ __forceinline__ void hier_nc_potential_warp(const float* z, float* g, double* __restrict__ pe_out,
                                                       int J, const float* __restrict__ y,
                                                       const float* __restrict__ sinv, double cmodel, float inv_ms2,
                                                       float inv_ts, int lane) {
  const float mu = z[0], lt = z[1];
  const float tau = expf(lt);
  float lpf = 0.0f, swf = 0.0f, swef = 0.0f;
  for (int j = lane; j < J; j += 32) {
    const float eta = z[2 + j];
    const float is = sinv[j];
    const float th = fmaf(tau, eta, mu);
    const float r = (y[j] - th) * is;
    lpf += -0.5f * eta * eta - 0.5f * r * r;
    const float w = r * is;
    swf += w;
    swef = fmaf(w, eta, swef);
    g[2 + j] = eta - tau * w;
  }
  FF flp = ff_from(lpf), fsw = ff_from(swf), fswe = ff_from(swef);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    flp = ff_add(flp, ff_shfl_xor(flp, o));
    fsw = ff_add(fsw, ff_shfl_xor(fsw, o));
    fswe = ff_add(fswe, ff_shfl_xor(fswe, o));
  }
  if (lane == 0) {
    const float sw = fsw.hi + fsw.lo, swe = fswe.hi + fswe.lo;
    const float u = tau * inv_ts;
    const float u2 = u * u;
    const float lp_prior = -0.5f * mu * mu * inv_ms2 - log1pf(u2) + lt;  // Normal(mu), HalfCauchy(tau) + log-det
    *pe_out = -(ff_value(flp) + (double)lp_prior - cmodel);
    g[0] = mu * inv_ms2 - sw;
    g[1] = 2.0f * u2 / (1.0f + u2) - 1.0f - tau * swe;
  }
}

}  // namespace gbn
