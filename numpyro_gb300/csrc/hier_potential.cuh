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

__device__ __forceinline__ void hier_nc_potential_warp(const float* z, float* g,
                                                       double* __restrict__ pe_out, int J,
                                                       const float* __restrict__ y, const float* __restrict__ sg,
                                                       double mu_scale, double tau_scale, int lane) {
  constexpr double LOG_2PI = 1.8378770664093453;
  constexpr double LOG_PI = 1.1447298858494002;
  constexpr double LOG_2 = 0.6931471805599453;
  const float mu = z[0], lt = z[1];
  const float tau = expf(lt);
  // per-lane partial sums in FP32 (at most 8 terms for J <= 256), summed across the warp as
  // float-float pairs
  float lpf = 0.0f, swf = 0.0f, swef = 0.0f;
  for (int j = lane; j < J; j += 32) {
    const float eta = z[2 + j];
    const float yy = y[j], s = sg[j];
    const float th = fmaf(tau, eta, mu);
    const float r = (yy - th) / s;
    lpf += -0.5f * eta * eta - 0.5f * r * r - logf(s);
    const float w = r / s;
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
  const double lp = ff_value(flp), sw = ff_value(fsw), swe = ff_value(fswe);
  if (lane == 0) {
    const double dmu = (double)mu, dt = exp((double)lt);
    const double lp_mu = -0.5 * (dmu / mu_scale) * (dmu / mu_scale) - 0.5 * LOG_2PI - log(mu_scale);
    const double lp_tau = -LOG_PI - log(tau_scale) - log1p((dt / tau_scale) * (dt / tau_scale)) + LOG_2 + (double)lt;
    const double total = lp + lp_mu + lp_tau - (double)J * LOG_2PI;  // two N(.) normalisers per group
    *pe_out = -total;
    g[0] = (float)(dmu / (mu_scale * mu_scale) - sw);
    g[1] = (float)(2.0 * dt * dt / (tau_scale * tau_scale + dt * dt) - 1.0 - dt * swe);
  }
}

}  // namespace gbn
