"""The oracle's potentials pinned to scipy.stats, and its analytic gradients to central differences.

Each potential is numpyro's potential_energy (numpyro/infer/util.py:333-358): minus the sum of
the sites' log-densities at the constrained values, minus log|det J| of the Exp transforms of
positive sites (transforms.py:641-644).  Here every log-density comes from scipy.stats, written
independently of oracle/potentials_ref.py, on seeded inputs:
  Normal continuous.py:2975-2989, HalfCauchy :1149-1150, HalfNormal :1190-1191,
  Exponential :715-726, StudentT :3229-3238, GaussianRandomWalk :1104-1112,
  BernoulliLogits discrete.py:263.
"""
import numpy as np
import pytest
from scipy import special, stats

from oracle import potentials_ref as PR


def _rng(seed):
    return np.random.default_rng(seed)


def _hier_case(seed):
    r = _rng(seed)
    J = 8
    y = r.normal(0, 10, J)
    sigma = r.uniform(9, 18, J)
    z = np.concatenate([[r.normal(0, 3)], [r.normal(0, 1)], r.normal(0, 1, J)])
    return z, (y, sigma)


def _hier_scipy(z, y, sigma):
    mu, ltau, eta = z[0], z[1], z[2:]
    tau = np.exp(ltau)
    lp = stats.norm.logpdf(mu, 0, 5) + stats.halfcauchy.logpdf(tau, scale=5) + ltau
    lp += stats.norm.logpdf(eta).sum() + stats.norm.logpdf(y, mu + tau * eta, sigma).sum()
    return -lp


def _logreg_case(seed):
    r = _rng(seed)
    X = np.concatenate([r.normal(size=(300, 6)), np.ones((300, 1))], axis=1)
    y = (r.random(300) < 0.4).astype(np.float64)
    return 0.4 * r.normal(size=7), (X, y)


def _logreg_scipy(b, X, y):
    return -(stats.bernoulli.logpmf(y, special.expit(X @ b)).sum() + stats.norm.logpdf(b).sum())


def _hs_case(seed, P=12, N=40):
    r = _rng(seed)
    X = r.normal(size=(N, P))
    y = X[:, 0] * 2.0 - X[:, 3] + r.normal(size=N)
    z = np.concatenate([r.normal(0, 1, P), r.normal(0, 0.5, P), [r.normal(0, 0.3)], [r.normal(0, 0.5)]])
    return z, (X, y)


def _hs_scipy(z, X, y):
    P = X.shape[1]
    beta, llam, lsig, ltau = z[:P], z[P:2 * P], z[2 * P], z[2 * P + 1]
    lam, sig, tau = np.exp(llam), np.exp(lsig), np.exp(ltau)
    lp = stats.norm.logpdf(beta, 0, tau * lam).sum()
    lp += stats.halfcauchy.logpdf(lam).sum() + llam.sum()
    lp += stats.halfnorm.logpdf(sig) + lsig + stats.halfcauchy.logpdf(tau) + ltau
    lp += stats.norm.logpdf(y, X @ beta, sig).sum()
    return -lp


def _hs_nc_scipy(z, X, y):
    P = X.shape[1]
    llam, lsig, ltau, eta = z[:P], z[P], z[P + 1], z[P + 2:]
    lam, sig, tau = np.exp(llam), np.exp(lsig), np.exp(ltau)
    lp = stats.norm.logpdf(eta).sum()
    lp += stats.halfcauchy.logpdf(lam).sum() + llam.sum()
    lp += stats.halfnorm.logpdf(sig) + lsig + stats.halfcauchy.logpdf(tau) + ltau
    lp += stats.norm.logpdf(y, X @ (tau * lam * eta), sig).sum()
    return -lp


def _sv_case(seed, T=64):
    r = _rng(seed)
    s, nu = 0.05, 8.0
    h = np.log(0.01) + np.cumsum(s * r.normal(size=T))
    ret = np.exp(h) * r.standard_t(nu, size=T)
    z = np.concatenate([h + 0.01 * r.normal(size=T), [np.log(nu) + 0.1], [np.log(s) - 0.1]])
    return z, (ret,)


def _sv_scipy(z, ret, s_rate=10.0, nu_rate=0.1):
    T = ret.shape[0]
    h, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = np.exp(lnu), np.exp(ls)
    lp = stats.expon.logpdf(s, scale=1 / s_rate) + ls + stats.expon.logpdf(nu, scale=1 / nu_rate) + lnu
    lp += stats.norm.logpdf(h[0], 0, s) + stats.norm.logpdf(np.diff(h), 0, s).sum()
    lp += stats.t.logpdf(ret, df=nu, loc=0, scale=np.exp(h)).sum()
    return -lp


def _sv_nc_case(seed, T=64):
    r = _rng(seed)
    ret = 0.01 * r.standard_t(8.0, size=T)
    z = np.concatenate([0.3 * r.normal(size=T), [np.log(8.0)], [np.log(0.05)]])
    return z, (ret,)


def _sv_nc_scipy(z, ret, s_rate=10.0, nu_rate=0.1):
    T = ret.shape[0]
    e, lnu, ls = z[:T], z[T], z[T + 1]
    nu, s = np.exp(lnu), np.exp(ls)
    h = s * np.cumsum(e)
    lp = stats.expon.logpdf(s, scale=1 / s_rate) + ls + stats.expon.logpdf(nu, scale=1 / nu_rate) + lnu
    lp += stats.norm.logpdf(e).sum() + stats.t.logpdf(ret, df=nu, loc=0, scale=np.exp(h)).sum()
    return -lp


CASES = {
    "hier_nc": (_hier_case, _hier_scipy),
    "logreg": (_logreg_case, _logreg_scipy),
    "horseshoe": (_hs_case, _hs_scipy),
    "horseshoe_nc": (_hs_case, _hs_nc_scipy),
    "sv": (_sv_case, _sv_scipy),
    "sv_nc": (_sv_nc_case, _sv_nc_scipy),
}


@pytest.mark.parametrize("family", sorted(CASES))
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_potential_matches_scipy_log_densities(family, seed):
    make_case, scipy_u = CASES[family]
    z, data = make_case(seed)
    pot, _ = PR.FAMILIES[family]
    u = pot(z, *data)
    ref = scipy_u(z, *data)
    assert abs(u - ref) <= 1e-10 * max(1.0, abs(ref)), (family, u, ref)


@pytest.mark.parametrize("family", sorted(CASES))
@pytest.mark.parametrize("seed", [0, 1])
def test_gradient_matches_central_differences(family, seed):
    make_case, _ = CASES[family]
    z, data = make_case(seed)
    pot, grad = PR.FAMILIES[family]
    g = grad(z, *data)
    fd = PR.central_fd_grad(lambda v: pot(v, *data), z, h=1e-5)
    scale = max(1.0, np.max(np.abs(fd)))
    np.testing.assert_allclose(g, fd, rtol=0, atol=1e-6 * scale)
