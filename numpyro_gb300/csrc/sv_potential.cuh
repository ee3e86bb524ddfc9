// sv_potential.cuh -- CTA-level potentials + adjoints of the stochastic-volatility
// family, shared by the tick-engine kernel (potentials_simt.cu) and the
// persistent engine (nuts_engine.cu) so that both produce bit-identical results.
//
//   s ~ Exponential(s_rate); nu ~ Exponential(nu_rate)        (Exp transforms, log-dets ls, lnu)
//   centred:      h ~ GaussianRandomWalk(scale=s, num_steps=T), z = [h(T), lnu, ls]
//   non-centred:  h_base ~ Normal(0, 1)^T, h = s * cumsum(h_base), z = [h_base(T), lnu, ls]
//   r_t ~ StudentT(nu, 0, exp(h_t))
// Log-densities: Exponential numpyro/distributions/continuous.py:715-726, GaussianRandomWalk
// :1104-1112, StudentT :3229-3238, Normal :2975-2989; Exp log-det transforms.py:641-644; model as
// examples/stochastic_volatility.py:58-66.
//
// Non-centred adjoint.  With S_t = sum_{k<=t} h_base_k and a_t = d log p(r_t | h_t) / d h_t,
//   dU/dh_base_k = h_base_k - s * sum_{t>=k} a_t,   dU/dls = -s * sum_t a_t S_t + s_rate * s - 1.
// Each thread owns one contiguous chunk of ceil(T/NT) steps.  The forward pass needs S_t: the
// walk is stored only at chunk starts (one checkpoint per thread, from a block-wide exclusive scan
// of the chunk totals) and recomputed inside the chunk from its checkpoint.  The reverse pass
// needs the suffix sums of a_t: a block-wide reverse exclusive scan of the chunk totals gives each
// thread its starting suffix; a_t itself stays in registers between the passes (or, for chunks
// too long for registers, is parked in the gradient row).  Running sums inside a chunk are compensated FP32
// (two-sum, Knuth TAOCP vol. 2 4.2.2); chunk totals are scanned and reduced as float-float
// pairs.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "common.cuh"

namespace gbn {

constexpr double SV_LOG_2PI = 1.8378770664093453;
constexpr double SV_LOG_PI = 1.1447298858494002;

// Scratch a CTA needs in shared memory for the SV potentials.
template <int NT>
struct SvSmem {
  double red[16];        // Group<256> reductions
  double special[9];     // lgamma(nu/2), lgamma((nu+1)/2), digamma(nu/2), digamma((nu+1)/2),
                         // nu, 1/nu, s, 1/s, log(s_rate) + log(nu_rate)
  float2 warp_tot[2][NT / 32];
};

// The scalar factors of the potential, each group on lane 0 of its own warp so they run side by
// side with the element loop; thread 0 reads them after the reductions' barriers.  The two
// log-gamma values enter U multiplied by T and grow like x log x, so they stay FP64 (in FP32,
// T * lgamma(nu/2) rounds to O(1) at large nu and roughens the energy surface).  The digammas
// enter only through a difference of order 1/nu in the gradient, and the remaining factors need
// no more than FP32 (GB300 issues FP64 at a small fraction of the FP32 rate).
template <int NT>
__device__ __forceinline__ void sv_special_functions(float lnuf, float lsf, double s_rate, double nu_rate, int tid,
                                                     double* special) {
  static_assert(NT >= 256, "needs six warps");
  if ((tid & 31) != 0) return;
  const float nu = expf(lnuf);
  switch (tid >> 5) {
    case 0: special[0] = lgamma(0.5 * (double)nu); break;
    case 1: special[1] = lgamma(0.5 * ((double)nu + 1.0)); break;
    case 2: special[2] = (double)digamma_f(0.5f * nu); break;
    case 3: special[3] = (double)digamma_f(0.5f * (nu + 1.0f)); break;
    case 4: special[4] = (double)nu; special[5] = (double)(1.0f / nu); break;
    case 5: {
      const float s = expf(lsf);
      special[6] = (double)s;
      special[7] = (double)(1.0f / s);
      special[8] = (double)(logf((float)s_rate) + logf((float)nu_rate));
      break;
    }
    default: break;
  }
}

// d/dlnu of U (both parameterisations): nu-dependent StudentT terms summed over T plus the prior.
__device__ __forceinline__ float sv_grad_lnu(double S_l1p, double S_frac, double T, double nu_rate,
                                             const double* special) {
  const double nu = special[4], inv_nu = special[5];
  double dnu = -0.5 * S_l1p + 0.5 * (nu + 1.0) * inv_nu * S_frac - 0.5 * T * inv_nu - 0.5 * T * special[2] +
               0.5 * T * special[3] - nu_rate;
  return (float)(-(dnu * nu + 1.0));
}

// The potentials are compiled out of line: the tick and persistent kernels then run one and
// the same instruction sequence (inlined into different kernels, floating-point contraction
// could differ between them and break their bit-identity).
// Centred GRW.  z/g are the chain's rows; pe_out is written by thread 0.
template <int NT>
__device__ __noinline__ void sv_potential_block(const float* z, float* g, double* pe_out, int T,
                                                   const float* __restrict__ ret, double s_rate, double nu_rate,
                                                   int tid, SvSmem<NT>& sm) {
  Group<NT> grp{tid};
  // FP32 nu and 1/s^2 for the element loop; FP64 nu and s only where the scalar terms need them
  const float lnuf = z[T], lsf = z[T + 1];
  const float nuf = expf(lnuf), sf = expf(lsf);
  const float inv_s2 = 1.0f / (sf * sf), inv_nuf = 1.0f / nuf;
  sv_special_functions<NT>(lnuf, lsf, s_rate, nu_rate, tid, sm.special);
  Comp32 sdd{0.0f, 0.0f}, sl1p{0.0f, 0.0f}, sfrac{0.0f, 0.0f}, sh{0.0f, 0.0f};
  constexpr int U = 4;  // loads of U steps are issued before their gradient stores
  for (int t0 = tid; t0 < T; t0 += U * NT) {
    float hv[U], hp[U], hn[U], rv[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int t = t0 + k * NT;
      const bool in = t < T;
      hv[k] = in ? z[t] : 0.0f;
      hp[k] = (in && t > 0) ? z[t - 1] : 0.0f;
      hn[k] = (t + 1 < T) ? z[t + 1] : 0.0f;
      rv[k] = in ? ret[t] : 0.0f;
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const int t = t0 + k * NT;
      if (t >= T) continue;
      const float h = hv[k];
      const float dprev = (t == 0) ? h : h - hp[k];
      const float dnext = (t + 1 < T) ? hn[k] - h : 0.0f;
      const float yv = rv[k] * expf(-h);
      const float y2 = yv * yv;
      const float q = y2 * inv_nuf;
      const float frac = __fdividef(y2, nuf + y2);
      sdd.add(dprev * dprev);
      sl1p.add(log1pf(q));
      sfrac.add(frac);
      sh.add(h);
      g[t] = (dprev - dnext) * inv_s2 + 1.0f - (nuf + 1.0f) * frac;
    }
  }
  FF f_dd = comp_ff(sdd), f_l1p = comp_ff(sl1p), f_frac = comp_ff(sfrac), f_h = comp_ff(sh);
  grp.sum2ff(f_dd, f_l1p, sm.red);
  grp.sum2ff(f_frac, f_h, sm.red);
  if (tid == 0) {
    const double lnu = lnuf, ls = lsf, nu = sm.special[4], s = sm.special[6], inv_s = sm.special[7];
    double S_dd = ff_value(f_dd), S_l1p = ff_value(f_l1p), S_frac = ff_value(f_frac), S_h = ff_value(f_h);
    double lp = sm.special[8] - s_rate * s + ls - nu_rate * nu + lnu;
    lp += -0.5 * S_dd * (inv_s * inv_s) - (double)T * ls - 0.5 * (double)T * SV_LOG_2PI;
    double zc = 0.5 * lnu + 0.5 * SV_LOG_PI + sm.special[0] - sm.special[1];
    lp += -0.5 * (nu + 1.0) * S_l1p - S_h - (double)T * zc;
    *pe_out = -lp;
    g[T] = sv_grad_lnu(S_l1p, S_frac, (double)T, nu_rate, sm.special);
    double ds = S_dd * (inv_s * inv_s * inv_s) - (double)T * inv_s - s_rate;
    g[T + 1] = (float)(-(ds * s + 1.0));
  }
}

// Block-wide exclusive scans of one float-float pair per thread (forward: sum over lower
// threads; reverse: sum over higher threads).  Lanes combine by shuffles, warps through `wt`
// (NT/32 pairs); each contains two barriers.
template <int NT>
__device__ __forceinline__ FF block_excl_scan(FF v, int tid, float2* wt) {
  const int lane = tid & 31, w = tid >> 5;
  FF excl{0.0f, 0.0f};
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {  // inclusive lane scan of v, then shift by one lane
    FF x{__shfl_up_sync(0xffffffffu, v.hi, o), __shfl_up_sync(0xffffffffu, v.lo, o)};
    if (lane >= o) v = ff_add(x, v);
  }
  excl.hi = __shfl_up_sync(0xffffffffu, v.hi, 1);
  excl.lo = __shfl_up_sync(0xffffffffu, v.lo, 1);
  if (lane == 0) excl = FF{0.0f, 0.0f};
  if (lane == 31) wt[w] = make_float2(v.hi, v.lo);
  __syncthreads();
  FF off{0.0f, 0.0f};
  for (int k = 0; k < w; ++k) off = ff_add(off, FF{wt[k].x, wt[k].y});
  __syncthreads();
  return ff_add(off, excl);
}
template <int NT>
__device__ __forceinline__ FF block_excl_rscan(FF v, int tid, float2* wt) {
  const int lane = tid & 31, w = tid >> 5;
  FF excl{0.0f, 0.0f};
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    FF x{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    if (lane + o < 32) v = ff_add(v, x);
  }
  excl.hi = __shfl_down_sync(0xffffffffu, v.hi, 1);
  excl.lo = __shfl_down_sync(0xffffffffu, v.lo, 1);
  if (lane == 31) excl = FF{0.0f, 0.0f};
  if (lane == 0) wt[w] = make_float2(v.hi, v.lo);
  __syncthreads();
  FF off{0.0f, 0.0f};
  for (int k = NT / 32 - 1; k > w; --k) off = ff_add(off, FF{wt[k].x, wt[k].y});
  __syncthreads();
  return ff_add(off, excl);
}

// Non-centred GRW (h = s * cumsum(h_base)).  z/g are the chain's rows.  Chunks of at most
// SV_REG_CHUNK steps (T <= 4096 with 256 threads) are held in registers.
constexpr int SV_REG_CHUNK = 16;
template <int NT>
__device__ __noinline__ void sv_nc_potential_block(const float* z, float* g, double* pe_out, int T,
                                                      const float* __restrict__ ret, double s_rate,
                                                      double nu_rate, int tid, SvSmem<NT>& sm) {
  Group<NT> grp{tid};
  const float lnuf = z[T], lsf = z[T + 1];
  const float nuf = expf(lnuf), sf = expf(lsf), inv_nuf = 1.0f / nuf;
  sv_special_functions<NT>(lnuf, lsf, s_rate, nu_rate, tid, sm.special);
  const int chunk = (T + NT - 1) / NT;
  const int t0 = min(T, tid * chunk), t1 = min(T, t0 + chunk);
  Comp32 sl1p{0.0f, 0.0f}, sfrac{0.0f, 0.0f}, sh{0.0f, 0.0f}, sas{0.0f, 0.0f}, se2{0.0f, 0.0f},
      atot{0.0f, 0.0f};
  // one step of the forward pass: extend the walk, accumulate, return a_t
  auto forward_step = [&](Comp32& S, float e, float r) -> float {
    S.add(e);
    const float St = S.value();
    const float h = sf * St;
    const float yv = r * expf(-h);
    const float y2 = yv * yv;
    const float frac = __fdividef(y2, nuf + y2);
    const float at = (nuf + 1.0f) * frac - 1.0f;  // d log p(r_t | h_t) / d h_t
    sl1p.add(log1pf(y2 * inv_nuf));
    sfrac.add(frac);
    sh.add(h);
    sas.add(at * St);
    se2.add(e * e);
    atot.add(at);
    return at;
  };
  if (chunk <= SV_REG_CHUNK) {
    // the chunk's h_base, returns and a_t stay in registers between the passes
    float ev[SV_REG_CHUNK], rv[SV_REG_CHUNK], av[SV_REG_CHUNK];
#pragma unroll
    for (int i = 0; i < SV_REG_CHUNK; ++i) {
      const bool in = t0 + i < t1;
      ev[i] = in ? z[t0 + i] : 0.0f;
      rv[i] = in ? ret[t0 + i] : 0.0f;
    }
    // chunk total of h_base -> checkpoint S_{t0-1} (exclusive scan)
    Comp32 tot{0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < SV_REG_CHUNK; ++i)
      if (t0 + i < t1) tot.add(ev[i]);
    const FF ck = block_excl_scan<NT>(comp_ff(tot), tid, sm.warp_tot[0]);
    Comp32 S{ck.hi, ck.lo};
#pragma unroll
    for (int i = 0; i < SV_REG_CHUNK; ++i) av[i] = (t0 + i < t1) ? forward_step(S, ev[i], rv[i]) : 0.0f;
    // reverse pass: suffix sums of a_t from the thread's starting suffix
    const FF suf = block_excl_rscan<NT>(comp_ff(atot), tid, sm.warp_tot[1]);
    Comp32 A{suf.hi, suf.lo};
#pragma unroll
    for (int i = SV_REG_CHUNK - 1; i >= 0; --i) {
      if (t0 + i >= t1) continue;
      A.add(av[i]);
      g[t0 + i] = ev[i] - sf * A.value();
    }
  } else {
    // long walks: a_t is parked in the gradient row between the passes
    Comp32 tot{0.0f, 0.0f};
    for (int t = t0; t < t1; ++t) tot.add(z[t]);
    const FF ck = block_excl_scan<NT>(comp_ff(tot), tid, sm.warp_tot[0]);
    Comp32 S{ck.hi, ck.lo};
    for (int t = t0; t < t1; ++t) g[t] = forward_step(S, z[t], ret[t]);
    const FF suf = block_excl_rscan<NT>(comp_ff(atot), tid, sm.warp_tot[1]);
    Comp32 A{suf.hi, suf.lo};
    for (int t = t1 - 1; t >= t0; --t) {
      A.add(g[t]);
      g[t] = z[t] - sf * A.value();
    }
  }
  FF f_l1p = comp_ff(sl1p), f_frac = comp_ff(sfrac), f_h = comp_ff(sh), f_as = comp_ff(sas);
  grp.sum2ff(f_l1p, f_frac, sm.red);
  grp.sum2ff(f_h, f_as, sm.red);
  const FF f_e2 = grp.sumff(comp_ff(se2), sm.red);
  if (tid == 0) {
    const double lnu = lnuf, ls = lsf, nu = sm.special[4], s = sm.special[6];
    double S_l1p = ff_value(f_l1p), S_frac = ff_value(f_frac), S_h = ff_value(f_h), S_as = ff_value(f_as),
           S_e2 = ff_value(f_e2);
    double lp = sm.special[8] - s_rate * s + ls - nu_rate * nu + lnu;
    lp += -0.5 * S_e2 - 0.5 * (double)T * SV_LOG_2PI;
    double zc = 0.5 * lnu + 0.5 * SV_LOG_PI + sm.special[0] - sm.special[1];
    lp += -0.5 * (nu + 1.0) * S_l1p - S_h - (double)T * zc;
    *pe_out = -lp;
    g[T] = sv_grad_lnu(S_l1p, S_frac, (double)T, nu_rate, sm.special);
    g[T + 1] = (float)(-s * S_as + s_rate * s - 1.0);
  }
}

}  // namespace gbn
