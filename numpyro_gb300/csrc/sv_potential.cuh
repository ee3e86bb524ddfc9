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
// thread its starting suffix, and a_t itself is parked in the gradient row (the only T-length
// buffer touched) between the passes.  Running sums inside a chunk are compensated FP32
// (two-sum, Knuth TAOCP vol. 2 4.2.2); chunk totals are scanned and reduced in FP64.
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
  double special[4];     // lgamma(nu/2), lgamma((nu+1)/2), digamma(nu/2), digamma((nu+1)/2)
  double warp_tot[2][NT / 32];
};

// The four FP64 special functions of nu, each on lane 0 of its own warp so they run side by side
// with the element loop; read after the next barrier.
template <int NT>
__device__ __forceinline__ void sv_special_functions(double nu, int tid, double* special) {
  static_assert(NT >= 128, "needs four warps");
  if (tid == 0) special[0] = lgamma(0.5 * nu);
  else if (tid == 32) special[1] = lgamma(0.5 * (nu + 1.0));
  else if (tid == 64) special[2] = digamma_d(0.5 * nu);
  else if (tid == 96) special[3] = digamma_d(0.5 * (nu + 1.0));
}

// d/dlnu of U (both parameterisations): nu-dependent StudentT terms summed over T plus the prior.
__device__ __forceinline__ float sv_grad_lnu(double nu, double S_l1p, double S_frac, double T, double nu_rate,
                                             const double* special) {
  double dnu = -0.5 * S_l1p + 0.5 * (nu + 1.0) / nu * S_frac - 0.5 * T / nu - 0.5 * T * special[2] +
               0.5 * T * special[3] - nu_rate;
  return (float)(-(dnu * nu + 1.0));
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

// Each thread's share of the T-length sums is accumulated in compensated FP32 and the shares
// are summed across the CTA in FP64.
__device__ __forceinline__ double comp_total(const Comp32& a) { return (double)a.s + (double)a.c; }

// The potentials are compiled out of line: the tick and persistent kernels then run one and
// the same instruction sequence (inlined into different kernels, floating-point contraction
// could differ between them and break their bit-identity).
// Centred GRW.  z/g are the chain's rows; pe_out is written by thread 0.
template <int NT>
__device__ __noinline__ void sv_potential_block(const float* z, float* g, double* pe_out, int T,
                                                   const float* __restrict__ ret, double s_rate, double nu_rate,
                                                   int tid, SvSmem<NT>& sm) {
  Group<NT> grp{tid};
  double lnu = z[T], ls = z[T + 1];
  double nu = exp(lnu), s = exp(ls);
  sv_special_functions<NT>(nu, tid, sm.special);
  float nuf = (float)nu;
  float inv_s2 = (float)(1.0 / (s * s));
  Comp32 sdd{0.0f, 0.0f}, sl1p{0.0f, 0.0f}, sfrac{0.0f, 0.0f}, sh{0.0f, 0.0f};
  for (int t = tid; t < T; t += NT) {
    float h = z[t];
    float dprev = (t == 0) ? h : h - z[t - 1];
    float dnext = (t + 1 < T) ? z[t + 1] - h : 0.0f;
    float rt = ret[t];
    float yv = rt * expf(-h);
    float y2 = yv * yv;
    float q = y2 / nuf;
    float frac = y2 / (nuf + y2);
    sdd.add(dprev * dprev);
    sl1p.add(log1pf(q));
    sfrac.add(frac);
    sh.add(h);
    g[t] = (dprev - dnext) * inv_s2 + 1.0f - (nuf + 1.0f) * frac;
  }
  double2 a = grp.sum2(make_double2(comp_total(sdd), comp_total(sl1p)), sm.red);
  double2 b = grp.sum2(make_double2(comp_total(sfrac), comp_total(sh)), sm.red);
  if (tid == 0) {
    double S_dd = a.x, S_l1p = a.y, S_frac = b.x, S_h = b.y;
    double lp = log(s_rate) - s_rate * s + ls;
    lp += log(nu_rate) - nu_rate * nu + lnu;
    lp += -0.5 * S_dd / (s * s) - (double)T * ls - 0.5 * (double)T * SV_LOG_2PI;
    double zc = 0.5 * lnu + 0.5 * SV_LOG_PI + sm.special[0] - sm.special[1];
    lp += -0.5 * (nu + 1.0) * S_l1p - S_h - (double)T * zc;
    *pe_out = -lp;
    g[T] = sv_grad_lnu(nu, S_l1p, S_frac, (double)T, nu_rate, sm.special);
    double ds = S_dd / (s * s * s) - (double)T / s - s_rate;
    g[T + 1] = (float)(-(ds * s + 1.0));
  }
}

// Block-wide exclusive scans of one double per thread (forward: sum over lower threads;
// reverse: sum over higher threads).  Contain two barriers; `wt` holds NT/32 doubles.
template <int NT>
__device__ __forceinline__ double block_excl_scan(double v, int tid, double* wt) {
  const int lane = tid & 31, w = tid >> 5;
  double incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    double x = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += x;
  }
  if (lane == 31) wt[w] = incl;
  __syncthreads();
  double off = 0.0;
  for (int k = 0; k < w; ++k) off += wt[k];
  __syncthreads();
  return off + incl - v;
}
template <int NT>
__device__ __forceinline__ double block_excl_rscan(double v, int tid, double* wt) {
  const int lane = tid & 31, w = tid >> 5;
  double incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    double x = __shfl_down_sync(0xffffffffu, incl, o);
    if (lane + o < 32) incl += x;
  }
  if (lane == 0) wt[w] = incl;
  __syncthreads();
  double off = 0.0;
  for (int k = NT / 32 - 1; k > w; --k) off += wt[k];
  __syncthreads();
  return off + incl - v;
}

// Non-centred GRW (h = s * cumsum(h_base)).  z/g are the chain's rows.
template <int NT>
__device__ __noinline__ void sv_nc_potential_block(const float* z, float* g, double* pe_out, int T,
                                                      const float* __restrict__ ret, double s_rate,
                                                      double nu_rate, int tid, SvSmem<NT>& sm) {
  Group<NT> grp{tid};
  double lnu = z[T], ls = z[T + 1];
  double nu = exp(lnu), s = exp(ls);
  sv_special_functions<NT>(nu, tid, sm.special);
  const float nuf = (float)nu, sf = (float)s;
  const int chunk = (T + NT - 1) / NT;
  const int t0 = min(T, tid * chunk), t1 = min(T, t0 + chunk);
  // chunk total of h_base -> checkpoint S_{t0-1} (exclusive scan)
  Comp32 tot{0.0f, 0.0f};
  for (int t = t0; t < t1; ++t) tot.add(z[t]);
  double ck = block_excl_scan<NT>(comp_total(tot), tid, sm.warp_tot[0]);
  // forward pass: recompute the walk from the checkpoint, park a_t in g
  Comp32 S{(float)ck, (float)(ck - (double)(float)ck)};
  Comp32 sl1p{0.0f, 0.0f}, sfrac{0.0f, 0.0f}, sh{0.0f, 0.0f}, sas{0.0f, 0.0f}, se2{0.0f, 0.0f},
      atot{0.0f, 0.0f};
  for (int t = t0; t < t1; ++t) {
    const float e = z[t];
    S.add(e);
    const float St = S.value();
    const float h = sf * St;
    const float yv = ret[t] * expf(-h);
    const float y2 = yv * yv;
    const float frac = y2 / (nuf + y2);
    const float at = (nuf + 1.0f) * frac - 1.0f;  // d log p(r_t | h_t) / d h_t
    sl1p.add(log1pf(y2 / nuf));
    sfrac.add(frac);
    sh.add(h);
    sas.add(at * St);
    se2.add(e * e);
    atot.add(at);
    g[t] = at;
  }
  // reverse pass: suffix sums of a_t from the thread's starting suffix
  const double suf = block_excl_rscan<NT>(comp_total(atot), tid, sm.warp_tot[1]);
  Comp32 A{(float)suf, (float)(suf - (double)(float)suf)};
  for (int t = t1 - 1; t >= t0; --t) {
    A.add(g[t]);
    g[t] = z[t] - sf * A.value();
  }
  double2 r1 = grp.sum2(make_double2(comp_total(sl1p), comp_total(sfrac)), sm.red);
  double2 r2 = grp.sum2(make_double2(comp_total(sh), comp_total(sas)), sm.red);
  double r3 = grp.sum(comp_total(se2), sm.red);
  if (tid == 0) {
    double S_l1p = r1.x, S_frac = r1.y, S_h = r2.x, S_as = r2.y, S_e2 = r3;
    double lp = log(s_rate) - s_rate * s + ls;
    lp += log(nu_rate) - nu_rate * nu + lnu;
    lp += -0.5 * S_e2 - 0.5 * (double)T * SV_LOG_2PI;
    double zc = 0.5 * lnu + 0.5 * SV_LOG_PI + sm.special[0] - sm.special[1];
    lp += -0.5 * (nu + 1.0) * S_l1p - S_h - (double)T * zc;
    *pe_out = -lp;
    g[T] = sv_grad_lnu(nu, S_l1p, S_frac, (double)T, nu_rate, sm.special);
    g[T + 1] = (float)(-s * S_as + s_rate * s - 1.0);
  }
}

}  // namespace gbn
