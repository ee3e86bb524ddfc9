/*
 * nuts_ref.c -- C restatement of numpyro's NUTS transition and warmup
 * (ORACLE / CPU BASELINE: test infrastructure, never linked into the product).
 *
 * Follows numpyro/infer/hmc_util.py: velocity_verlet :262-311,
 * _build_basetree :851-894, _combine_tree :767-848, _iterative_build_subtree
 * :984-1085, _leaf_idx_to_ckpt_idxs :941-958, _is_iterative_turning
 * :961-981, build_tree :1088-1180, dual_averaging :60-130,
 * welford_covariance :133-239, build_adaptation_schedule :387-436,
 * warmup_adapter :518-707; numpyro/infer/hmc.py sample_kernel :459-530.
 * Potentials follow numpyro's potential_energy (numpyro/infer/util.py:333-358)
 * for the registry families, as oracle/potentials_ref.py restates them (which
 * the CPU tests pin to scipy.stats and to central differences; this file is
 * pinned to that restatement by tests/test_oracle_c.py).
 * Randomness: Philox4x32-10 at the stream addresses of oracle/philox.py.
 *
 * Build: REAL=double (FP64 oracle) or REAL=float (FP32, numpyro's default
 * dtype; sums accumulate in double).  OpenMP runs independent chains in
 * parallel (the CPU analogue of chain_method="parallel").
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef REAL
#define REAL double
#endif
#ifndef REAL_IS_FLOAT
#define REAL_IS_FLOAT 0
#endif
typedef REAL real;

#define LOG_2PI 1.8378770664093453
#define LOG_PI 1.1447298858494002
#define LOG_2 0.6931471805599453

/* ------------------------------------------------------------------ Philox */
static void philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct { uint32_t lo, hi; } seed_t;
enum { P_MOMENTUM = 0, P_DOUBLING = 1, P_LEAF = 2, P_INIT = 3 };

static void draw(seed_t s, uint32_t chain, uint32_t n, uint32_t purpose, uint32_t idx, uint32_t sub, uint32_t o[4]) {
  uint32_t c[4] = {chain, n, (purpose << 24) | idx, sub};
  philox(c, s.lo, s.hi, o);
}
static double u01(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }

static void normals(seed_t s, uint32_t chain, uint32_t n, uint32_t purpose, int dim, real* out) {
  for (int k = 0; 4 * k < dim; ++k) {
    uint32_t w[4];
    draw(s, chain, n, purpose, (uint32_t)k, 0, w);
    for (int pr = 0; pr < 2; ++pr) {
      double u0 = u01(w[2 * pr]), u1 = u01(w[2 * pr + 1]);
      double rad = sqrt(-2.0 * log1p(-u0)), ang = 2.0 * M_PI * u1;
      int d0 = 4 * k + 2 * pr;
      if (d0 < dim) out[d0] = (real)(rad * cos(ang));
      if (d0 + 1 < dim) out[d0 + 1] = (real)(rad * sin(ang));
    }
  }
}

/* ------------------------------------------------------------------ models */
/* The registry model (mirrors gbn_model_desc of include/gbnuts.h):
 *   family 1  non-centred hierarchical normal; N groups in num_models datasets (offsets),
 *             chain c runs dataset c / chains_per_model; hyper = (mu scale, tau scale)
 *   family 2  logistic regression, X [N][P]; hyper[0] = prior scale
 *   family 3  horseshoe regression, X [N][P]; hyper[0] = 1 selects the non-centred form
 *   family 4  stochastic volatility, returns y [N = T]; hyper = (s rate, nu rate, non-centred) */
typedef struct {
  int32_t family;
  int32_t num_models;
  int32_t chains_per_model;
  int32_t P;
  int64_t N;
  const float* X;
  const float* y;
  const float* sigma;
  const int32_t* offsets;
  double hyper[4];
  int32_t row_threads; /* logistic family: threads sharing one chain's rows (0/1: none) */
  double target_accept; /* dual-averaging target accept probability (0: numpyro's default 0.8) */
} nutsref_model;

int nutsref_latent_dim(const nutsref_model* m, int model_index) {
  switch (m->family) {
    case 1:
      if (m->offsets) return m->offsets[model_index + 1] - m->offsets[model_index] + 2;
      return (int)m->N + 2;
    case 2: return m->P;
    case 3: return 2 * m->P + 2;
    case 4: return (int)m->N + 2;
    default: return 0;
  }
}

static int model_of_chain(const nutsref_model* m, uint32_t chain) {
  if (m->family != 1 || !m->offsets) return 0;
  int cpm = m->chains_per_model > 0 ? m->chains_per_model : 1;
  int k = (int)(chain / (uint32_t)cpm);
  return k < m->num_models ? k : m->num_models - 1;
}

/* digamma: upward recurrence to x >= 10, then the asymptotic series
 * psi(x) ~ ln x - 1/(2x) - sum_k B_2k / (2k x^2k) (Abramowitz & Stegun 6.3.18) */
static double digamma_ref(double x) {
  double acc = 0.0;
  while (x < 10.0) {
    acc -= 1.0 / x;
    x += 1.0;
  }
  double f = 1.0 / (x * x);
  double t = f * (-1.0 / 12 + f * (1.0 / 120 + f * (-1.0 / 252 + f * (1.0 / 240 + f * (-1.0 / 132 +
             f * (691.0 / 32760 + f * (-1.0 / 12)))))));
  return acc + log(x) - 0.5 / x + t;
}

#if REAL_IS_FLOAT
/* FP32 transcendentals written so a compiler can vectorise the row loop (libm calls would stay
 * scalar), as XLA's CPU backend does for numpyro's float32 potential:
 *   exp: Cody & Waite (1980) range reduction x = k ln2 + r, |r| <= ln2/2, with the degree-6 Taylor
 *        polynomial of e^r (truncation error 0.347^7 / 7! = 1.2e-7 relative);
 *   log1p: log(1 + t) = 2 atanh(s), s = t / (2 + t) in [0, 1/3] for t in [0, 1], by the odd series
 *        2 (s + s^3/3 + ... + s^13/13) (Abramowitz & Stegun 4.1.28; truncation error < 2e-8). */
static inline float exp_neg_f(float x) { /* e^x for x <= 0 */
  x = x < -87.0f ? -87.0f : x;
  /* k = round(x log2 e): x <= 0, so truncating x log2 e - 1/2 toward zero rounds to nearest
   * (the build reassociates float sums, so an add-and-subtract rounding trick would fold away) */
  const int32_t ki = (int32_t)(x * 1.44269504088896341f - 0.5f);
  const float kf = (float)ki;
  const float r = (x - kf * 0.693145751953125f) - kf * 1.428606765330187e-06f;
  float p = 1.0f / 720.0f;
  p = p * r + 1.0f / 120.0f;
  p = p * r + 1.0f / 24.0f;
  p = p * r + 1.0f / 6.0f;
  p = p * r + 0.5f;
  p = p * r + 1.0f;
  p = p * r + 1.0f;
  union { float f; int32_t i; } u;
  u.i = (ki + 127) << 23;
  return p * u.f;
}
static inline float log1p_unit_f(float t) { /* log(1 + t) for t in [0, 1] */
  const float s = t / (2.0f + t), s2 = s * s;
  float q = 1.0f / 13.0f;
  q = q * s2 + 1.0f / 11.0f;
  q = q * s2 + 1.0f / 9.0f;
  q = q * s2 + 1.0f / 7.0f;
  q = q * s2 + 1.0f / 5.0f;
  q = q * s2 + 1.0f / 3.0f;
  q = q * s2 + 1.0f;
  return 2.0f * s * q;
}
#endif

/* numpyro potential_energy of the logistic model (examples/covtype.py:66-71): rows [n0, n1) into
 * double partials ga (gradient of the log-likelihood part) and *ll; per-row arithmetic in `real`,
 * blocks of LR_BLOCK rows flushed into the double accumulators. */
#define LR_BLOCK 256
static void logreg_rows(const nutsref_model* m, const real* b, int64_t r0, int64_t r1, double* ga, double* ll) {
  const int D = m->P;
  real gb[64];
  real lb[LR_BLOCK], eb[LR_BLOCK];
  double lls = 0.0;
  for (int d = 0; d < D; ++d) gb[d] = 0;
  for (int64_t n0 = r0; n0 < r1; n0 += LR_BLOCK) {
    const int nb = (int)(n0 + LR_BLOCK < r1 ? LR_BLOCK : r1 - n0);
    const float* xb = m->X + n0 * D;
    for (int r = 0; r < nb; ++r) {
      const float* x = xb + (int64_t)r * D;
      real l = 0;
#pragma omp simd reduction(+ : l)
      for (int d = 0; d < D; ++d) l += (real)x[d] * b[d];
      lb[r] = l;
    }
    real llb = 0;
#if REAL_IS_FLOAT
#pragma omp simd reduction(+ : llb)
    for (int r = 0; r < nb; ++r) {
      const real l = lb[r], yy = (real)m->y[n0 + r];
      const real t = exp_neg_f(-fabsf(l));
      const real sp = (l > 0 ? l : 0.0f) + log1p_unit_f(t);
      const real inv = 1.0f / (1.0f + t);
      const real sig = l >= 0 ? inv : t * inv;
      llb += sp - yy * l;
      eb[r] = sig - yy;
    }
#else
    for (int r = 0; r < nb; ++r) {
      const real l = lb[r], yy = (real)m->y[n0 + r];
      const real t = exp(-fabs(l));
      const real sp = (l > 0 ? l : 0.0) + log1p(t);
      const real sig = l >= 0 ? (real)1 / ((real)1 + t) : t / ((real)1 + t);
      llb += sp - yy * l;
      eb[r] = sig - yy;
    }
#endif
    for (int r = 0; r < nb; ++r) {
      const float* x = xb + (int64_t)r * D;
      const real e = eb[r];
#pragma omp simd
      for (int d = 0; d < D; ++d) gb[d] += e * (real)x[d];
    }
    /* block partial sums (<= 256 rows) are flushed into double accumulators */
    lls += (double)llb;
    for (int d = 0; d < D; ++d) {
      ga[d] += (double)gb[d];
      gb[d] = 0;
    }
  }
  *ll += lls;
}

/* With row_threads > 1 the rows are split into that many contiguous ranges evaluated by an OpenMP
 * team (the chains then run one after another), and the ranges' partials are added in order. */
static double logreg_pg(const nutsref_model* m, const real* b, real* g) {
  const int D = m->P;
  double ll = 0.0;
  double ga[64];
  for (int d = 0; d < D; ++d) ga[d] = 0.0;
  const int T = m->row_threads > 1 ? m->row_threads : 1;
  if (T == 1) {
    logreg_rows(m, b, 0, m->N, ga, &ll);
  } else {
    double part[T][65];
#pragma omp parallel num_threads(T)
    {
#ifdef _OPENMP
      const int k = omp_get_thread_num(), nt = omp_get_num_threads();
#else
      const int k = 0, nt = 1;
#endif
      const int64_t per = (m->N + T - 1) / T;
      for (int kk = k; kk < T; kk += nt) {
        double* pp = part[kk];
        for (int d = 0; d <= D; ++d) pp[d] = 0.0;
        const int64_t a = (int64_t)kk * per, e = a + per < m->N ? a + per : m->N;
        if (a < e) logreg_rows(m, b, a, e, pp, &pp[D]);
      }
    }
    for (int kk = 0; kk < T; ++kk) {
      for (int d = 0; d < D; ++d) ga[d] += part[kk][d];
      ll += part[kk][D];
    }
  }
  double pr = 0.0, s = m->hyper[0] > 0 ? m->hyper[0] : 1.0;
  for (int d = 0; d < D; ++d) {
    g[d] = (real)(ga[d] + (double)b[d] / (s * s));
    pr += 0.5 * (double)b[d] * (double)b[d] / (s * s) + 0.5 * log(2 * M_PI) + log(s);
  }
  return ll + pr;
}

/* non-centred hierarchical normal of dataset k, z = [mu, log tau, theta_base(J)]
 * (potentials_ref.hier_nc_potential / hier_nc_grad) */
static double hier_pg(const nutsref_model* m, int k, const real* z, real* g) {
  int j0 = m->offsets ? m->offsets[k] : 0;
  int J = m->offsets ? m->offsets[k + 1] - j0 : (int)m->N;
  const float* ys = m->y + j0;
  const float* ss = m->sigma + j0;
  double ms = m->hyper[0] > 0 ? m->hyper[0] : 5.0, ts = m->hyper[1] > 0 ? m->hyper[1] : 5.0;
  double mu = z[0], lt = z[1], tau = exp(lt);
  double lp = -0.5 * (mu / ms) * (mu / ms) - 0.5 * log(2 * M_PI) - log(ms);
  lp += -log(M_PI) - log(ts) - log1p((tau / ts) * (tau / ts)) + log(2.0) + lt;
  double sw = 0, swe = 0;
  for (int j = 0; j < J; ++j) {
    double eta = z[2 + j], s = ss[j], th = mu + tau * eta, r = (ys[j] - th) / s;
    lp += -0.5 * eta * eta - 0.5 * r * r - log(s) - log(2 * M_PI);
    double w = r / s;
    sw += w;
    swe += w * eta;
    g[2 + j] = (real)(eta - tau * w);
  }
  g[0] = (real)(mu / (ms * ms) - sw);
  g[1] = (real)(2 * tau * tau / (ts * ts + tau * tau) - 1 - tau * swe);
  return -lp;
}

/* Horseshoe regression (potentials_ref.horseshoe_* / horseshoe_nc_*), FP64 arithmetic.
 * centred:     z = [beta(P), log lambda(P), log sigma, log tau]
 * non-centred: z = [log lambda(P), log sigma, log tau, unscaled_betas(P)], beta = tau lambda eta */
static double horseshoe_pg(const nutsref_model* m, const real* z, real* g) {
  const int P = m->P;
  const int64_t N = m->N;
  const int nc = m->hyper[0] != 0.0;
  const real* llam = nc ? z : z + P;
  const double lsig = nc ? z[P] : z[2 * P], ltau = nc ? z[P + 1] : z[2 * P + 1];
  const double sig = exp(lsig), tau = exp(ltau);
  double* beta = (double*)malloc(sizeof(double) * (size_t)P);
  double* gx = (double*)calloc((size_t)P, sizeof(double));
  for (int d = 0; d < P; ++d) beta[d] = nc ? tau * exp((double)llam[d]) * (double)z[P + 2 + d] : (double)z[d];
  double rr = 0.0;
  for (int64_t n = 0; n < N; ++n) {
    const float* x = m->X + n * P;
    double acc = 0.0;
#pragma omp simd reduction(+ : acc)
    for (int d = 0; d < P; ++d) acc += (double)x[d] * beta[d];
    const double r = (double)m->y[n] - acc;
    rr += r * r;
    for (int d = 0; d < P; ++d) gx[d] += r * (double)x[d];
  }
  const double inv_s2 = 1.0 / (sig * sig);
  for (int d = 0; d < P; ++d) gx[d] *= inv_s2; /* -dU_lik/dbeta */
  double lp = 0.0;
  /* likelihood: Normal(resid; 0, sigma) */
  lp += -0.5 * rr * inv_s2 - (double)N * (0.5 * LOG_2PI + lsig);
  /* sigma ~ HalfNormal(1) with its Exp log-det */
  lp += -0.5 * sig * sig - 0.5 * LOG_2PI + LOG_2 + lsig;
  /* tau ~ HalfCauchy(1) */
  lp += -LOG_PI - log1p(tau * tau) + LOG_2 + ltau;
  double gtau = 0.0;
  for (int d = 0; d < P; ++d) {
    const double ll = llam[d], lam = exp(ll);
    lp += -LOG_PI - log1p(lam * lam) + LOG_2 + ll; /* lambda_d ~ HalfCauchy(1) */
    if (nc) {
      const double eta = z[P + 2 + d];
      lp += -0.5 * eta * eta - 0.5 * LOG_2PI;
      g[P + 2 + d] = (real)(eta - tau * lam * gx[d]);
      g[d] = (real)(-beta[d] * gx[d] + 2.0 * lam * lam / (1.0 + lam * lam) - 1.0);
      gtau += -beta[d] * gx[d];
    } else {
      const double s = tau * lam, b = beta[d], q = b * b / (s * s);
      lp += -0.5 * q - 0.5 * LOG_2PI - log(s);
      g[d] = (real)(b / (s * s) - gx[d]);
      g[P + d] = (real)(-q + 2.0 * lam * lam / (1.0 + lam * lam));
      gtau += -q + 1.0;
    }
  }
  const int is = nc ? P : 2 * P;
  g[is] = (real)(sig * sig - 1.0 - rr * inv_s2 + (double)N);
  g[is + 1] = (real)(gtau + 2.0 * tau * tau / (1.0 + tau * tau) - 1.0);
  free(beta);
  free(gx);
  return -lp;
}

/* Stochastic volatility (potentials_ref.sv_* / sv_nc_*), FP64 arithmetic.
 * centred:     z = [h(T), log nu, log s], h ~ GaussianRandomWalk(s)
 * non-centred: z = [h_base(T), log nu, log s], h = s cumsum(h_base) */
static double sv_pg(const nutsref_model* m, const real* z, real* g) {
  const int T = (int)m->N;
  const double s_rate = m->hyper[0] > 0 ? m->hyper[0] : 10.0, nu_rate = m->hyper[1] > 0 ? m->hyper[1] : 0.1;
  const int nc = m->hyper[2] != 0.0;
  const double lnu = z[T], ls = z[T + 1], nu = exp(lnu), s = exp(ls);
  double lp = log(s_rate) - s_rate * s + ls + log(nu_rate) - nu_rate * nu + lnu;
  const double zc = 0.5 * lnu + 0.5 * LOG_PI + lgamma(0.5 * nu) - lgamma(0.5 * (nu + 1.0));
  const double dig = -0.5 / nu - 0.5 * digamma_ref(0.5 * nu) + 0.5 * digamma_ref(0.5 * (nu + 1.0));
  double dlp_dnu = 0.0, sumsq = 0.0, as = 0.0, cum = 0.0;
  double* a = (double*)malloc(sizeof(double) * (size_t)T);
  double* S = (double*)malloc(sizeof(double) * (size_t)T);
  for (int t = 0; t < T; ++t) {
    double h;
    if (nc) {
      cum += (double)z[t];
      S[t] = cum;
      h = s * cum;
      lp += -0.5 * (double)z[t] * (double)z[t] - 0.5 * LOG_2PI;
    } else {
      h = z[t];
      const double d = t == 0 ? (double)z[0] : (double)z[t] - (double)z[t - 1];
      sumsq += d * d;
    }
    const double yv = (double)m->y[t] * exp(-h), y2 = yv * yv;
    lp += -0.5 * (nu + 1.0) * log1p(y2 / nu) - (h + zc);
    a[t] = (nu + 1.0) * y2 / (nu + y2) - 1.0; /* d log StudentT / d h_t */
    dlp_dnu += -0.5 * log1p(y2 / nu) + 0.5 * (nu + 1.0) * y2 / (nu * (nu + y2)) + dig;
  }
  if (!nc) lp += -0.5 * sumsq / (s * s) - (double)T * (0.5 * LOG_2PI + ls);
  dlp_dnu += -nu_rate;
  g[T] = (real)(-(dlp_dnu * nu + 1.0));
  if (nc) {
    double suffix = 0.0;
    for (int t = T - 1; t >= 0; --t) {
      suffix += a[t];
      g[t] = (real)((double)z[t] - s * suffix);
      as += a[t] * S[t];
    }
    g[T + 1] = (real)(-s * as + s_rate * s - 1.0);
  } else {
    const double is2 = 1.0 / (s * s);
    for (int t = 0; t < T; ++t) {
      double gh = 0.0;
      const double dprev = t == 0 ? (double)z[0] : (double)z[t] - (double)z[t - 1];
      gh += dprev * is2;
      if (t + 1 < T) gh -= ((double)z[t + 1] - (double)z[t]) * is2;
      g[t] = (real)(gh - a[t]);
    }
    const double dlp_ds = sumsq / (s * s * s) - (double)T / s - s_rate;
    g[T + 1] = (real)(-(dlp_ds * s + 1.0));
  }
  free(a);
  free(S);
  return -lp;
}

static double potential_grad(const nutsref_model* m, int k, const real* z, real* g) {
  switch (m->family) {
    case 1: return hier_pg(m, k, z, g);
    case 2: return logreg_pg(m, z, g);
    case 3: return horseshoe_pg(m, z, g);
    default: return sv_pg(m, z, g);
  }
}

/* U and dU/dz of one latent point of dataset model_index (FP64 in and out). */
double nutsref_potential(const nutsref_model* m, int model_index, const double* z, double* g) {
  int D = nutsref_latent_dim(m, model_index);
  real* zr = (real*)malloc(sizeof(real) * (size_t)D);
  real* gr = (real*)malloc(sizeof(real) * (size_t)D);
  for (int d = 0; d < D; ++d) zr[d] = (real)z[d];
  double pe = potential_grad(m, model_index, zr, gr);
  for (int d = 0; d < D; ++d) g[d] = (double)gr[d];
  free(zr);
  free(gr);
  return pe;
}

/* ------------------------------------------------------------------ chain */
typedef struct {
  int D, maxd, k; /* latent dim, checkpoint rows, dataset index */
  real *z, *g, *inv, *msq;
  real *zl, *rl, *gl, *zr, *rr, *gr, *zp, *gp, *zsp, *gsp, *rs, *rss, *rck, *sck, *tmp;
  double pe, step, ss[5], target_accept;
  double *mean, *m2;
  int mm_n, window_idx;
  long grad_evals;
} chain_t;

static void chain_alloc(chain_t* c, int D, int maxd, int k) {
  c->D = D;
  c->maxd = maxd;
  c->k = k;
  real** vs[] = {&c->z, &c->g, &c->inv, &c->msq, &c->zl, &c->rl, &c->gl, &c->zr, &c->rr, &c->gr, &c->zp,
                 &c->gp, &c->zsp, &c->gsp, &c->rs, &c->rss, &c->tmp};
  for (size_t v = 0; v < sizeof(vs) / sizeof(vs[0]); ++v) *vs[v] = (real*)calloc((size_t)D, sizeof(real));
  c->rck = (real*)calloc((size_t)maxd * D, sizeof(real));
  c->sck = (real*)calloc((size_t)maxd * D, sizeof(real));
  c->mean = (double*)calloc((size_t)D, sizeof(double));
  c->m2 = (double*)calloc((size_t)D, sizeof(double));
}

static void chain_free(chain_t* c) {
  real** vs[] = {&c->z, &c->g, &c->inv, &c->msq, &c->zl, &c->rl, &c->gl, &c->zr, &c->rr, &c->gr, &c->zp,
                 &c->gp, &c->zsp, &c->gsp, &c->rs, &c->rss, &c->tmp};
  for (size_t v = 0; v < sizeof(vs) / sizeof(vs[0]); ++v) free(*vs[v]);
  free(c->rck); free(c->sck); free(c->mean); free(c->m2);
}

static double kinetic(const chain_t* c, const real* r) {
  double k = 0;
  for (int d = 0; d < c->D; ++d) k += (double)c->inv[d] * (double)r[d] * (double)r[d];
  return 0.5 * k;
}

static int is_turning(const chain_t* c, const real* rl, const real* rr, const real* rs, const real* rsm,
                      const real* rsp) {
  double a = 0, b = 0;
  for (int d = 0; d < c->D; ++d) {
    double s = rs[d];
    if (rsm) s = s - rsm[d] + rsp[d];
    s -= 0.5 * ((double)rl[d] + (double)rr[d]);
    a += (double)c->inv[d] * rl[d] * s;
    b += (double)c->inv[d] * rr[d] * s;
  }
  return a <= 0 || b <= 0;
}

static double logaddexp(double a, double b) {
  double mx = a > b ? a : b;
  if (mx == -INFINITY) return -INFINITY;
  return mx + log1p(exp(-fabs(a - b)));
}

/* one leapfrog from the frontier (z, r, g) in place; returns pe */
static double leapfrog(const nutsref_model* m, chain_t* c, real* z, real* r, real* g, double eps) {
  for (int d = 0; d < c->D; ++d) {
    r[d] = (real)((double)r[d] - 0.5 * eps * g[d]);
    z[d] = (real)((double)z[d] + eps * (double)c->inv[d] * r[d]);
  }
  double pe = potential_grad(m, c->k, z, g);
  c->grad_evals++;
  for (int d = 0; d < c->D; ++d) r[d] = (real)((double)r[d] - 0.5 * eps * g[d]);
  return pe;
}

/* One NUTS transition (hmc.py:459-530 with build_tree hmc_util.py:1088-1180). */
static void nuts_transition(const nutsref_model* m, chain_t* c, seed_t s, uint32_t chain, uint32_t n, int max_depth,
                            int* num_steps, double* accept_prob, int* diverging) {
  int D = c->D;
  real* r0 = c->tmp;
  normals(s, chain, n, P_MOMENTUM, D, r0);
  for (int d = 0; d < D; ++d) r0[d] *= c->msq[d];
  double e0 = c->pe + kinetic(c, r0);
  memcpy(c->zl, c->z, D * sizeof(real)); memcpy(c->zr, c->z, D * sizeof(real)); memcpy(c->zp, c->z, D * sizeof(real));
  memcpy(c->gl, c->g, D * sizeof(real)); memcpy(c->gr, c->g, D * sizeof(real)); memcpy(c->gp, c->g, D * sizeof(real));
  memcpy(c->rl, r0, D * sizeof(real)); memcpy(c->rr, r0, D * sizeof(real)); memcpy(c->rs, r0, D * sizeof(real));
  int depth = 0, turning = 0, div = 0, nprop = 0;
  double tw = 0, tacc = 0, pe_p = c->pe;
  while (depth < max_depth && !turning && !div) {
    uint32_t w[4];
    draw(s, chain, n, P_DOUBLING, (uint32_t)depth, 0, w);
    int right = u01(w[0]) < 0.5;
    double eps = right ? c->step : -c->step;
    real *zf = right ? c->zr : c->zl, *rf = right ? c->rr : c->rl, *gf = right ? c->gr : c->gl;
    int snum = 0, sdiv = 0, sturn = 0, maxn = 1 << depth;
    double sw = 0, sacc = 0, pe_sp = 0;
    while (snum < maxn && !sturn && !sdiv) {
      double pe = leapfrog(m, c, zf, rf, gf, eps);
      double dE = pe + kinetic(c, rf) - e0;
      if (isnan(dE)) dE = INFINITY;
      double lw = -dE, acc = exp(-dE) < 1 ? exp(-dE) : 1.0;
      int leaf = snum;
      if (leaf == 0) {
        memcpy(c->zsp, zf, D * sizeof(real)); memcpy(c->gsp, gf, D * sizeof(real)); memcpy(c->rss, rf, D * sizeof(real));
        sw = lw; pe_sp = pe; sacc = acc;
      } else {
        uint32_t u[4];
        draw(s, chain, n, P_LEAF, (uint32_t)depth, (uint32_t)leaf, u);
        double p = 1.0 / (1.0 + exp(-(lw - sw)));
        if (u01(u[0]) < p) {
          memcpy(c->zsp, zf, D * sizeof(real)); memcpy(c->gsp, gf, D * sizeof(real));
          pe_sp = pe;
        }
        for (int d = 0; d < D; ++d) c->rss[d] += rf[d];
        sw = logaddexp(sw, lw);
        sacc += acc;
      }
      sdiv = dE > 1000.0;
      snum++;
      int idx_max = __builtin_popcount((unsigned)(leaf >> 1));
      int nsub = __builtin_popcount((unsigned)((~leaf & (leaf + 1)) - 1));
      int idx_min = idx_max - nsub + 1;
      if ((leaf & 1) == 0) {
        memcpy(c->rck + (size_t)idx_max * D, rf, D * sizeof(real));
        memcpy(c->sck + (size_t)idx_max * D, c->rss, D * sizeof(real));
      }
      for (int k = idx_max; k >= idx_min && !sturn; --k)
        sturn = is_turning(c, c->rck + (size_t)k * D, rf, c->rss, c->sck + (size_t)k * D, c->rck + (size_t)k * D);
    }
    for (int d = 0; d < D; ++d) c->rs[d] += c->rss[d];
    double p = (sturn || sdiv) ? 0.0 : (exp(sw - tw) < 1 ? exp(sw - tw) : 1.0);
    turning = sturn || is_turning(c, c->rl, c->rr, c->rs, NULL, NULL);
    if (u01(w[1]) < p) {
      memcpy(c->zp, c->zsp, D * sizeof(real)); memcpy(c->gp, c->gsp, D * sizeof(real));
      pe_p = pe_sp;
    }
    depth++;
    tw = logaddexp(tw, sw);
    div = sdiv;
    tacc += sacc;
    nprop += snum;
  }
  memcpy(c->z, c->zp, D * sizeof(real));
  memcpy(c->g, c->gp, D * sizeof(real));
  c->pe = pe_p;
  *num_steps = nprop;
  *accept_prob = tacc / nprop;
  *diverging = div;
}

static int window_ends(int num_steps, int* ends) {
  int k = 0;
  if (num_steps <= 0) return 0;
  if (num_steps < 20) { ends[k++] = num_steps - 1; return k; }
  int sb = 75, eb = 50, iw = 25;
  if (sb + eb + iw > num_steps) { sb = (int)(0.15 * num_steps); eb = (int)(0.1 * num_steps); iw = num_steps - sb - eb; }
  ends[k++] = sb - 1;
  int ews = num_steps - eb, ns = iw, nst = sb;
  while (nst < ews) {
    int cs = nst, cz = ns;
    if (3 * cz <= ews - cs) ns = 2 * cz; else cz = ews - cs;
    nst = cs + cz;
    ends[k++] = nst - 1;
  }
  ends[k++] = num_steps - 1;
  return k;
}

/* warmup_adapter.update_fn (hmc_util.py:637-705), diagonal mass, no heuristic */
static void adapt(chain_t* c, int t, double accept_prob, int num_warmup, const int* ends, int nwin) {
  double* ss = c->ss;
  ss[3] += 1.0;
  double tt = ss[3];
  ss[2] = (1 - 1 / (tt + 10)) * ss[2] + (c->target_accept - accept_prob) / (tt + 10);
  ss[0] = ss[4] - pow(tt, 0.5) / 0.05 * ss[2];
  double wt = pow(tt, -0.75);
  ss[1] = (1 - wt) * ss[1] + wt * ss[0];
  double st = (t == num_warmup - 1) ? exp(ss[1]) : exp(ss[0]);
  real sf = (real)st; /* step size carried in the build's precision */
  if (!(sf >= (real)1.17549435e-38)) sf = (real)1.17549435e-38;
  c->step = sf;
  int mid = (0 < c->window_idx) && (c->window_idx < nwin - 1);
  if (mid) {
    c->mm_n++;
    for (int d = 0; d < c->D; ++d) {
      double x = c->z[d], dp = x - c->mean[d];
      c->mean[d] += dp / c->mm_n;
      c->m2[d] += dp * (x - c->mean[d]);
    }
  }
  int at_end = c->window_idx < nwin && t == ends[c->window_idx];
  if (at_end) c->window_idx++;
  if (at_end && mid) {
    int nn = c->mm_n;
    for (int d = 0; d < c->D; ++d) {
      double cov = c->m2[d] / (nn - 1);
      cov = ((double)nn / (nn + 5.0)) * cov + 1e-3 * (5.0 / (nn + 5.0));
      c->inv[d] = (real)cov;
      c->msq[d] = (real)(1.0 / sqrt((double)(real)cov));
      c->mean[d] = 0; c->m2[d] = 0;
    }
    c->mm_n = 0;
    ss[0] = ss[1] = ss[2] = ss[3] = 0;
    ss[4] = log(10.0) + log(c->step);
  }
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/*
 * Replays one NUTS transition for each of `chains` chains from a given state, without
 * adaptation: chain k has global id chain_ids[k] (its Philox stream and, for the
 * hierarchical family, its dataset), transition counter iters[k], position z0 (row k of a
 * [chains][ld] array), step size step[k], and diagonal mass rows inv / msq ([chains][ld];
 * msq = mass_matrix_sqrt).  The potential at z0 is recomputed here.  Outputs: z_out
 * [chains][ld], num_steps, accept_prob, diverging, potential energy of the new state.
 */
int nutsref_transitions(const nutsref_model* m, int chains, const uint32_t* chain_ids, const uint32_t* iters, int ld,
                        const float* z0, const float* step, const float* inv, const float* msq, uint64_t seed,
                        int max_depth, int threads, float* z_out, int32_t* num_steps, double* accept_prob,
                        uint8_t* diverging, double* pe_out) {
  seed_t s = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) if (m->row_threads <= 1)
  for (int k = 0; k < chains; ++k) {
    chain_t c;
    memset(&c, 0, sizeof(c));
    const int mk = model_of_chain(m, chain_ids[k]);
    const int D = nutsref_latent_dim(m, mk);
    chain_alloc(&c, D, max_depth, mk);
    for (int d = 0; d < D; ++d) {
      c.z[d] = (real)z0[(size_t)k * ld + d];
      c.inv[d] = (real)inv[(size_t)k * ld + d];
      c.msq[d] = (real)msq[(size_t)k * ld + d];
    }
    c.step = (real)step[k];
    c.pe = potential_grad(m, mk, c.z, c.g);
    int ns = 0, dv = 0;
    double ap = 0.0;
    nuts_transition(m, &c, s, chain_ids[k], iters[k], max_depth, &ns, &ap, &dv);
    for (int d = 0; d < ld; ++d) z_out[(size_t)k * ld + d] = d < D ? (float)c.z[d] : 0.0f;
    num_steps[k] = ns;
    accept_prob[k] = ap;
    diverging[k] = (uint8_t)dv;
    pe_out[k] = c.pe;
    chain_free(&c);
  }
  return 0;
}

/*
 * Runs `chains` independent chains (ids first_chain..) for num_warmup + num_samples NUTS
 * transitions of model m.  If init_z is given ([chains][ld], with init_step/init_inv),
 * warmup adaptation is skipped and num_warmup transitions run without adaptation; else
 * init_to_uniform(radius=2) and the Stan warmup (dual averaging, diagonal Welford).
 * samples: [chains][num_samples][ld]; num_steps_out / diverging_out: [chains][num_samples];
 * adapted_step [chains] and adapted_inv [chains][ld] receive the state after warmup (may be NULL).
 * timing: [warmup_s, sampling_s, warmup_grad_evals, sampling_grad_evals, threads].
 */
int nutsref_run_model(const nutsref_model* m, int ld, int chains, int first_chain, int num_warmup, int num_samples,
                      uint64_t seed, int max_tree_depth, int threads, const float* init_z, const float* init_step,
                      const float* init_inv, float* samples, int32_t* num_steps_out, uint8_t* diverging_out,
                      float* adapted_step, float* adapted_inv, double* timing, double warmup_budget_s) {
  seed_t s = {(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32)};
  int ends[64];
  int nwin = window_ends(num_warmup, ends);
  double tw0 = 0, tw1 = 0, ts1 = 0;
  long gw = 0, gs = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#endif
  chain_t* cs = (chain_t*)calloc((size_t)chains, sizeof(chain_t));
  int maxd = max_tree_depth;
  for (int k = 0; k < chains; ++k) {
    chain_t* c = &cs[k];
    uint32_t chain = (uint32_t)(first_chain + k);
    const int mk = model_of_chain(m, chain);
    const int D = nutsref_latent_dim(m, mk);
    chain_alloc(c, D, maxd, mk);
    if (init_z) {
      for (int d = 0; d < D; ++d) {
        c->z[d] = init_z[(size_t)k * ld + d];
        c->inv[d] = init_inv[(size_t)k * ld + d];
        c->msq[d] = (real)(1.0 / sqrt((double)c->inv[d]));
      }
      c->step = init_step[k];
    } else {
      for (int b = 0; 4 * b < D; ++b) {
        uint32_t w[4];
        draw(s, chain, 0, P_INIT, (uint32_t)b, 0, w);
        for (int j = 0; j < 4 && 4 * b + j < D; ++j) c->z[4 * b + j] = (real)(-2.0 + 4.0 * u01(w[j]));
      }
      for (int d = 0; d < D; ++d) { c->inv[d] = 1; c->msq[d] = 1; }
      c->step = 1.0;
    }
    c->ss[4] = log(10.0 * c->step);
    c->target_accept = m->target_accept > 0 ? m->target_accept : 0.8;
  }
  tw0 = now_s();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : gw) if (m->row_threads <= 1)
  for (int k = 0; k < chains; ++k) {
    chain_t* c = &cs[k];
    c->pe = potential_grad(m, c->k, c->z, c->g);
    uint32_t chain = (uint32_t)(first_chain + k);
    for (int t = 0; t < num_warmup; ++t) {
      int ns, dv;
      double ap;
      /* a bounded baseline may cut the warmup short; it is reported as such */
      if (warmup_budget_s > 0 && now_s() - tw0 > warmup_budget_s) break;
      nuts_transition(m, c, s, chain, (uint32_t)t, max_tree_depth, &ns, &ap, &dv);
      if (!init_z) adapt(c, t, ap, num_warmup, ends, nwin);
    }
    gw += c->grad_evals;
    c->grad_evals = 0;
  }
  tw1 = now_s();
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : gs) if (m->row_threads <= 1)
  for (int k = 0; k < chains; ++k) {
    chain_t* c = &cs[k];
    uint32_t chain = (uint32_t)(first_chain + k);
    if (adapted_step) adapted_step[k] = (float)c->step;
    if (adapted_inv)
      for (int d = 0; d < ld; ++d) adapted_inv[(size_t)k * ld + d] = d < c->D ? (float)c->inv[d] : 0.0f;
    for (int t = 0; t < num_samples; ++t) {
      int ns, dv;
      double ap;
      nuts_transition(m, c, s, chain, (uint32_t)(num_warmup + t), max_tree_depth, &ns, &ap, &dv);
      for (int d = 0; d < ld; ++d)
        samples[((size_t)k * num_samples + t) * ld + d] = d < c->D ? (float)c->z[d] : 0.0f;
      if (num_steps_out) num_steps_out[(size_t)k * num_samples + t] = ns;
      if (diverging_out) diverging_out[(size_t)k * num_samples + t] = (uint8_t)dv;
    }
    gs += c->grad_evals;
  }
  ts1 = now_s();
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  timing[0] = tw1 - tw0;
  timing[1] = ts1 - tw1;
  timing[2] = (double)gw;
  timing[3] = (double)gs;
  timing[4] = (double)nthreads;
  for (int k = 0; k < chains; ++k) chain_free(&cs[k]);
  free(cs);
  return 0;
}

/* The logistic / eight-schools entry point of the CPU baseline (family 1 with one dataset of
 * N groups, or family 2 with P = D features); see nutsref_run_model. */
int nutsref_run(int family, const float* X, const float* y, const float* sigma, int64_t N, int D, double h0,
                double h1, int chains, int first_chain, int num_warmup, int num_samples, uint64_t seed,
                int max_tree_depth, int threads, const float* init_z, const float* init_step,
                const float* init_inv, float* samples, int32_t* num_steps_out, double* timing,
                double warmup_budget_s) {
  nutsref_model m;
  memset(&m, 0, sizeof(m));
  m.family = family;
  m.num_models = 1;
  m.chains_per_model = chains + first_chain;
  m.P = family == 2 ? D : 0;
  m.N = N;
  m.X = X;
  m.y = y;
  m.sigma = sigma;
  m.offsets = NULL;
  m.hyper[0] = h0;
  m.hyper[1] = h1;
  return nutsref_run_model(&m, D, chains, first_chain, num_warmup, num_samples, seed, max_tree_depth, threads,
                           init_z, init_step, init_inv, samples, num_steps_out, NULL, NULL, NULL, timing,
                           warmup_budget_s);
}
