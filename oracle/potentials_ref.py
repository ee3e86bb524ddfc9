"""FP64 potentials and analytic gradients (oracle side, test infrastructure).

A potential is numpyro's ``potential_energy`` (numpyro/infer/util.py:333-358):
the negative sum of every site's ``log_prob`` evaluated at the constrained
value, plus -log|det J| of each ``biject_to(support)`` transform
(infer/util.py:300-330).  Latent coordinates are laid out as
``ravel_pytree`` of the site dict, i.e. sites in sorted-name order, each site
in C order (hmc.py:101, hmc_util.py:186).

Log-densities restated here (numpyro/distributions):
  Normal        continuous.py:2975-2989   -0.5 ((x-m)/s)^2 - log(sqrt(2 pi) s)
  Cauchy        continuous.py:390-406     -log pi - log s - log1p(((x-m)/s)^2)
  HalfCauchy    continuous.py:1149-1150   Cauchy(0, s) + log 2
  HalfNormal    continuous.py:1190-1191   Normal(0, s) + log 2
  Exponential   continuous.py:715-726     log rate - rate x
  StudentT      continuous.py:3229-3238   -0.5 (nu+1) log1p(y^2/nu) - z,
                z = log s + 0.5 log nu + 0.5 log pi + lgamma(nu/2) - lgamma((nu+1)/2)
  GaussianRandomWalk continuous.py:1104-1112  Normal(0,s)(h_0) + sum_t Normal(0,s)(h_t - h_{t-1})
  BernoulliLogits discrete.py:263 + util.py:317-320  -(max(l,0) + log1p(exp(-|l|)) - l y)
Transforms: biject_to(positive) = ExpTransform (transforms.py:2115-2118),
log|det J| = x (transforms.py:641-644); biject_to(real/real_vector) = identity.
"""
import math

import numpy as np
from scipy.special import gammaln, digamma

LOG_2PI = math.log(2.0 * math.pi)
LOG_PI = math.log(math.pi)
LOG_2 = math.log(2.0)


def _normal_lp(x, loc, scale):
    return -0.5 * ((x - loc) / scale) ** 2 - math.log(math.sqrt(2 * math.pi)) - np.log(scale)


def _halfcauchy_lp(x, scale):
    return -LOG_PI - np.log(scale) - np.log1p((x / scale) ** 2) + LOG_2


# --------------------------------------------------------------------------
# Non-centred hierarchical normal ("eight schools" with TransformReparam):
#   mu ~ N(0, mu_scale); tau ~ HalfCauchy(tau_scale);
#   theta_base_j ~ N(0, 1); theta_j = mu + tau * theta_base_j (reparam.py:154-191)
#   y_j ~ N(theta_j, sigma_j)
# sorted sites: mu, tau, theta_base  ->  z = [mu, log tau, eta_1..eta_J]
# --------------------------------------------------------------------------
def hier_nc_potential(z, y, sigma, mu_scale=5.0, tau_scale=5.0):
    z = np.asarray(z, np.float64)
    mu, ltau, eta = z[0], z[1], z[2:]
    tau = math.exp(ltau)
    theta = mu + tau * eta
    lp = _normal_lp(mu, 0.0, mu_scale)
    lp += _halfcauchy_lp(tau, tau_scale) + ltau
    lp += np.sum(_normal_lp(eta, 0.0, 1.0))
    lp += np.sum(_normal_lp(y, theta, sigma))
    return -float(lp)


def hier_nc_grad(z, y, sigma, mu_scale=5.0, tau_scale=5.0):
    z = np.asarray(z, np.float64)
    mu, ltau, eta = z[0], z[1], z[2:]
    tau = math.exp(ltau)
    theta = mu + tau * eta
    w = (y - theta) / sigma ** 2  # d loglik / d theta
    g = np.empty_like(z)
    g[0] = mu / mu_scale ** 2 - np.sum(w)
    # d/dtau [-log HC] = 2 tau / (s^2 + tau^2); chain rule * tau; -1 for log-det
    g[1] = (2.0 * tau / (tau_scale ** 2 + tau ** 2)) * tau - 1.0 - tau * np.sum(w * eta)
    g[2:] = eta - tau * w
    return g


# --------------------------------------------------------------------------
# Bayesian logistic regression (examples/covtype.py:66-71):
#   coefs ~ N(0, 1)^D; obs ~ Bernoulli(logits = X coefs)
# --------------------------------------------------------------------------
def softplus(x):
    return np.maximum(x, 0.0) + np.log1p(np.exp(-np.abs(x)))


def logreg_potential(z, X, y):
    b = np.asarray(z, np.float64)
    logits = X @ b
    ll = -(softplus(logits) - logits * y)
    lp = np.sum(ll) + np.sum(_normal_lp(b, 0.0, 1.0))
    return -float(lp)


def logreg_grad(z, X, y):
    b = np.asarray(z, np.float64)
    logits = X @ b
    sig = 0.5 * (1.0 + np.tanh(0.5 * logits))
    return X.T @ (sig - y) + b


# --------------------------------------------------------------------------
# Horseshoe regression (centred), Gaussian likelihood:
#   tau ~ HalfCauchy(1); lambdas_d ~ HalfCauchy(1); beta_d ~ N(0, tau*lambda_d)
#   sigma ~ HalfNormal(1); y ~ N(X beta, sigma)
# sorted sites: beta, lambdas, sigma, tau -> z = [beta(P), log lambdas(P), log sigma, log tau]
# --------------------------------------------------------------------------
def horseshoe_unpack(z, P):
    z = np.asarray(z, np.float64)
    return z[:P], z[P:2 * P], z[2 * P], z[2 * P + 1]


def horseshoe_potential(z, X, y):
    P = X.shape[1]
    beta, llam, lsig, ltau = horseshoe_unpack(z, P)
    lam, sig, tau = np.exp(llam), math.exp(lsig), math.exp(ltau)
    lp = np.sum(_normal_lp(beta, 0.0, tau * lam))
    lp += np.sum(_halfcauchy_lp(lam, 1.0)) + np.sum(llam)
    lp += _normal_lp(sig, 0.0, 1.0) + LOG_2 + lsig
    lp += _halfcauchy_lp(tau, 1.0) + ltau
    resid = y - X @ beta
    lp += np.sum(_normal_lp(resid, 0.0, sig))
    return -float(lp)


def horseshoe_grad(z, X, y):
    N, P = X.shape
    beta, llam, lsig, ltau = horseshoe_unpack(z, P)
    lam, sig, tau = np.exp(llam), math.exp(lsig), math.exp(ltau)
    resid = y - X @ beta
    s = tau * lam
    g = np.empty(2 * P + 2)
    # prior on beta: 0.5 (b/s)^2 + log s
    g[:P] = beta / s ** 2 - X.T @ resid / sig ** 2
    # d/dlog lam of [0.5 b^2/(tau lam)^2 + log lam] = -b^2/s^2 + 1 ; HC(lam): 2 lam^2/(1+lam^2); logdet -1
    g[P:2 * P] = -(beta ** 2) / s ** 2 + 1.0 + 2.0 * lam ** 2 / (1.0 + lam ** 2) - 1.0
    # sigma: HalfNormal -> 0.5 sig^2 -> sig^2 ; logdet -1 ; likelihood 0.5 r^2/sig^2 + N log sig -> -r^2/sig^2 + N
    g[2 * P] = sig ** 2 - 1.0 - np.sum(resid ** 2) / sig ** 2 + N
    # tau: beta prior -> sum(-b^2/s^2 + 1); HC -> 2 tau^2/(1+tau^2); logdet -1
    g[2 * P + 1] = np.sum(-(beta ** 2) / s ** 2 + 1.0) + 2.0 * tau ** 2 / (1.0 + tau ** 2) - 1.0
    return g


# Non-centred horseshoe (examples/horseshoe_regression.py:33-49 with the HalfNormal(1) noise
# scale): sorted sites lambdas, sigma, tau, unscaled_betas -> z = [log lam(P), log sig, log tau, eta(P)],
# beta = tau * lam * eta, eta ~ Normal(0, 1).
def horseshoe_nc_potential(z, X, y):
    z = np.asarray(z, np.float64)
    P = X.shape[1]
    llam, lsig, ltau, eta = z[:P], z[P], z[P + 1], z[P + 2:]
    lam, sig, tau = np.exp(llam), math.exp(lsig), math.exp(ltau)
    beta = tau * lam * eta
    lp = np.sum(_normal_lp(eta, 0.0, 1.0))
    lp += np.sum(_halfcauchy_lp(lam, 1.0)) + np.sum(llam)
    lp += _normal_lp(sig, 0.0, 1.0) + LOG_2 + lsig
    lp += _halfcauchy_lp(tau, 1.0) + ltau
    lp += np.sum(_normal_lp(y - X @ beta, 0.0, sig))
    return -float(lp)


def horseshoe_nc_grad(z, X, y):
    z = np.asarray(z, np.float64)
    N, P = X.shape
    llam, lsig, ltau, eta = z[:P], z[P], z[P + 1], z[P + 2:]
    lam, sig, tau = np.exp(llam), math.exp(lsig), math.exp(ltau)
    beta = tau * lam * eta
    resid = y - X @ beta
    gx = X.T @ resid / sig ** 2                      # -dU_lik/dbeta
    g = np.empty(2 * P + 2)
    g[P + 2:] = eta - tau * lam * gx
    g[:P] = -beta * gx + 2.0 * lam ** 2 / (1.0 + lam ** 2) - 1.0
    g[P] = sig ** 2 - 1.0 - np.sum(resid ** 2) / sig ** 2 + N
    g[P + 1] = -np.sum(beta * gx) + 2.0 * tau ** 2 / (1.0 + tau ** 2) - 1.0
    return g


# --------------------------------------------------------------------------
# Stochastic volatility (examples/stochastic_volatility.py:58-66 with the
# Exponential(10) scale prior):  s ~ Exponential(10); nu ~ Exponential(0.1)
#   h ~ GaussianRandomWalk(scale=s, num_steps=T); r_t ~ StudentT(nu, 0, exp(h_t))
# sorted sites: h, nu, s -> z = [h(T), log nu, log s]
# --------------------------------------------------------------------------
def sv_potential(z, r, s_rate=10.0, nu_rate=0.1):
    z = np.asarray(z, np.float64)
    T = r.shape[0]
    h, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = math.exp(lnu), math.exp(ls)
    lp = math.log(s_rate) - s_rate * s + ls
    lp += math.log(nu_rate) - nu_rate * nu + lnu
    lp += _normal_lp(h[0], 0.0, s) + np.sum(_normal_lp(np.diff(h), 0.0, s))
    y = r * np.exp(-h)
    zt = h + 0.5 * lnu + 0.5 * LOG_PI + gammaln(0.5 * nu) - gammaln(0.5 * (nu + 1.0))
    lp += np.sum(-0.5 * (nu + 1.0) * np.log1p(y ** 2 / nu) - zt)
    return -float(lp)


def sv_grad(z, r, s_rate=10.0, nu_rate=0.1):
    z = np.asarray(z, np.float64)
    T = r.shape[0]
    h, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = math.exp(lnu), math.exp(ls)
    g = np.zeros(T + 2)
    d = np.diff(h)
    # GRW: 0.5 h0^2/s^2 + 0.5 sum d^2/s^2 + T log s
    gh = np.zeros(T)
    gh[0] += h[0] / s ** 2
    gh[1:] += d / s ** 2
    gh[:-1] -= d / s ** 2
    y2 = (r * np.exp(-h)) ** 2
    gh += 1.0 - (nu + 1.0) * y2 / (nu + y2)
    g[:T] = gh
    # nu: -[ -0.5 log1p(y2/nu) + 0.5 (nu+1) y2/(nu (nu + y2)) - 0.5/nu - 0.5 psi(nu/2) + 0.5 psi((nu+1)/2) ]
    dlp_dnu = np.sum(
        -0.5 * np.log1p(y2 / nu) + 0.5 * (nu + 1.0) * y2 / (nu * (nu + y2))
        - 0.5 / nu - 0.5 * digamma(0.5 * nu) + 0.5 * digamma(0.5 * (nu + 1.0))
    )
    dlp_dnu += -nu_rate
    g[T] = -(dlp_dnu * nu + 1.0)
    sumsq = h[0] ** 2 + np.sum(d ** 2)
    dlp_ds = sumsq / s ** 3 - T / s - s_rate
    g[T + 1] = -(dlp_ds * s + 1.0)
    return g


# Non-centred variant: sorted sites h_base, nu, s -> z = [h_base(T), log nu, log s],
# h = s * cumsum(h_base), h_base ~ Normal(0, 1)^T.
def sv_nc_potential(z, r, s_rate=10.0, nu_rate=0.1):
    z = np.asarray(z, np.float64)
    T = r.shape[0]
    e, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = math.exp(lnu), math.exp(ls)
    h = s * np.cumsum(e)
    lp = math.log(s_rate) - s_rate * s + ls
    lp += math.log(nu_rate) - nu_rate * nu + lnu
    lp += np.sum(_normal_lp(e, 0.0, 1.0))
    y = r * np.exp(-h)
    zt = h + 0.5 * lnu + 0.5 * LOG_PI + gammaln(0.5 * nu) - gammaln(0.5 * (nu + 1.0))
    lp += np.sum(-0.5 * (nu + 1.0) * np.log1p(y ** 2 / nu) - zt)
    return -float(lp)


def sv_nc_grad(z, r, s_rate=10.0, nu_rate=0.1):
    z = np.asarray(z, np.float64)
    T = r.shape[0]
    e, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = math.exp(lnu), math.exp(ls)
    S = np.cumsum(e)
    h = s * S
    y2 = (r * np.exp(-h)) ** 2
    a = (nu + 1.0) * y2 / (nu + y2) - 1.0          # d log StudentT(r_t | h_t) / d h_t
    suffix = np.cumsum(a[::-1])[::-1]               # sum_{t >= k} a_t
    g = np.zeros(T + 2)
    g[:T] = e - s * suffix
    dlp_dnu = np.sum(
        -0.5 * np.log1p(y2 / nu) + 0.5 * (nu + 1.0) * y2 / (nu * (nu + y2))
        - 0.5 / nu - 0.5 * digamma(0.5 * nu) + 0.5 * digamma(0.5 * (nu + 1.0))
    )
    dlp_dnu += -nu_rate
    g[T] = -(dlp_dnu * nu + 1.0)
    g[T + 1] = -s * np.sum(a * S) + s_rate * s - 1.0
    return g


FAMILIES = {
    "hier_nc": (hier_nc_potential, hier_nc_grad),
    "logreg": (logreg_potential, logreg_grad),
    "horseshoe": (horseshoe_potential, horseshoe_grad),
    "horseshoe_nc": (horseshoe_nc_potential, horseshoe_nc_grad),
    "sv": (sv_potential, sv_grad),
    "sv_nc": (sv_nc_potential, sv_nc_grad),
}


def make_potential(family, *data, **hyper):
    """Returns potential_fn(z) -> (pe, grad) closed over the data (FP64)."""
    pot, grad = FAMILIES[family]

    def potential_and_grad(z):
        return pot(z, *data, **hyper), grad(z, *data, **hyper)

    return potential_and_grad


def central_fd_grad(f, z, h=1e-3):
    z = np.asarray(z, np.float64)
    g = np.empty_like(z)
    for i in range(z.size):
        e = np.zeros_like(z)
        e[i] = h
        g[i] = (f(z + e) - f(z - e)) / (2 * h)
    return g
