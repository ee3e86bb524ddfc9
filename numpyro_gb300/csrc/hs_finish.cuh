// hs_finish.cuh -- the last step of the horseshoe regression potential for one point, by one
// 256-thread group: the prior terms and gradient per coordinate (FP32 with compensated sums, the
// scalar factors combined in FP64) from the GEMMs' partials X^T R (part_gb, split over row ranges)
// and sum R^2 (part_rr, per row tile).  Shared by the finish kernel and by the state-machine kernel
// that fuses it into the tick engine (a CTA per chain), so both give the same bits.
// (numpyro: examples/horseshoe_regression.py:33-49 -- HalfCauchy(1) tau and lambdas, Normal(0,
//  tau lambda) or the non-centred unscaled_betas ~ Normal(0, 1) with beta = tau lambda unscaled,
//  HalfNormal(1) sigma, Normal(X beta, sigma) likelihood; potential_energy infer/util.py:333-358.)
#pragma once
#include "common.cuh"

namespace gbn {

constexpr double HS_LOG_2PI = 1.8378770664093453;
constexpr double HS_LOG_PI = 1.1447298858494002;
constexpr double HS_LOG_2 = 0.6931471805599453;

__device__ __forceinline__ void horseshoe_finish_block(const float* __restrict__ Q, int c, int ld, int P, int64_t N,
                                                       const float* __restrict__ part_gb, int splits, int ldg,
                                                       int npts, const double* __restrict__ part_rr, int ld_rr,
                                                       int mtiles, int noncentred, double* __restrict__ PE,
                                                       float* __restrict__ G, int tid, double* red) {
  Group<256> g{tid};
  const float* z = Q + (size_t)c * ld;
  float* gz = G + (size_t)c * ld;
  const int i_sig = noncentred ? P : 2 * P, i_tau = i_sig + 1;
  const float lsig = z[i_sig], ltau = z[i_tau];
  const float inv_sig2 = expf(-2.0f * lsig);
  double rrd = 0.0;  // this thread's row tiles (at most a few), then a float-float pair
  for (int t = tid; t < mtiles; t += 256) rrd += part_rr[(size_t)t * ld_rr + c];
  const float rr_hi = (float)rrd;
  const FF rr_ff{rr_hi, (float)(rrd - (double)rr_hi)};
  Comp32 lp{0.0f, 0.0f}, gt{0.0f, 0.0f};
  for (int d = tid; d < P; d += 256) {
    float gb = 0.0f;
    for (int k = 0; k < splits; ++k) gb += part_gb[((size_t)k * npts + c) * ldg + d];
    const float gx = gb * inv_sig2;  // (X^T R)_d / sigma^2
    const float l = noncentred ? z[d] : z[P + d];
    const float e2 = expf(-2.0f * fabsf(l));
    const float log1p_lam2 = 2.0f * fmaxf(l, 0.0f) + log1pf(e2);
    const float hc = (l >= 0.0f) ? 2.0f / (1.0f + e2) : 2.0f * e2 / (1.0f + e2);  // 2 lam^2 / (1 + lam^2)
    if (noncentred) {
      const float eta = z[P + 2 + d];
      const float scale = expf(ltau + l);  // tau lambda_d
      const float bg = scale * eta * gx;   // beta_d g_d
      gz[P + 2 + d] = eta - scale * gx;
      gz[d] = hc - 1.0f - bg;
      lp.add(-0.5f * eta * eta - log1p_lam2 + l);
      gt.add(-bg);
    } else {
      const float b = z[d];
      const float inv_s2 = expf(-2.0f * (ltau + l));
      const float b2s = b * b * inv_s2;
      gz[d] = b * inv_s2 - gx;
      gz[P + d] = hc - b2s;
      lp.add(-0.5f * b2s - log1p_lam2);
      gt.add(1.0f - b2s);
    }
  }
  FF flp = comp_ff(lp), fgt = comp_ff(gt);
  g.sum2ff(flp, fgt, red);
  FF frr = g.sumff(rr_ff, red);
  if (tid == 0) {
    // The scalar factors come from FP32 transcendentals (correctly rounded to ~1 ulp) and are
    // combined in FP64 where a term is large (N log sigma, RR / sigma^2): an FP64 exp or log1p on
    // one thread costs microseconds on GB300's FP64 pipe, at the end of every chain's launch.
    const double RR = ff_value(frr), dlsig = lsig, dltau = ltau;
    const float sigf = expf(lsig), tauf = expf(ltau);
    const double sig = sigf, tau = tauf, inv_s2 = inv_sig2;
    // per coordinate: Normal(beta; 0, tau lambda) or Normal(unscaled; 0, 1), HalfCauchy(lambda; 1)
    double total = ff_value(flp) + (double)P * (HS_LOG_2 - HS_LOG_PI - 0.5 * HS_LOG_2PI - (noncentred ? 0.0 : dltau));
    total += -0.5 * sig * sig - 0.5 * HS_LOG_2PI + HS_LOG_2 + dlsig;  // HalfNormal(sigma; 1) + log-det
    total += -HS_LOG_PI - (double)log1pf(tauf * tauf) + HS_LOG_2 + dltau;  // HalfCauchy(tau; 1) + log-det
    total += -0.5 * RR * inv_s2 - (double)N * dlsig - 0.5 * (double)N * HS_LOG_2PI;
    PE[c] = -total;
    gz[i_sig] = (float)(sig * sig - 1.0 - RR * inv_s2 + (double)N);
    gz[i_tau] = (float)(ff_value(fgt) + (double)(2.0f * tauf * tauf / (1.0f + tauf * tauf)) - 1.0);
  }
}

}  // namespace gbn
