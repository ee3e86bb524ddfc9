"""Registry of model families with fused GPU potentials.

Each model states numpyro's site layout: sites in sorted-name order, each
flattened in C order (``ravel_pytree`` of the site dict, numpyro/infer/hmc.py:101,
numpyro/infer/hmc_util.py:186), and the ``biject_to(support)`` transform of
each site (Exp for positive sites, transforms.py:2115-2118; identity for real
and real_vector, :2143-2149, :2208-2210).  ``postprocess`` maps unconstrained
draws to constrained site values like numpyro's ``postprocess_fn``
(numpyro/infer/util.py:177-261).

Models written as numpyro programs (for reference):

  HierarchicalNormal (non-centred, TransformReparam, reparam.py:154-191)
      mu ~ Normal(0, mu_scale); tau ~ HalfCauchy(tau_scale)
      theta = mu + tau * theta_base, theta_base ~ Normal(0, 1)^J
      y_j ~ Normal(theta_j, sigma_j)
  LogisticRegression (examples/covtype.py:66-71)
      coefs ~ Normal(0, prior_scale)^D; obs ~ Bernoulli(logits = X coefs)
  HorseshoeRegression (Gaussian likelihood)
      tau ~ HalfCauchy(1); lambdas ~ HalfCauchy(1)^P; beta ~ Normal(0, tau*lambdas)
      sigma ~ HalfNormal(1); y ~ Normal(X beta, sigma)
      noncentered=True (examples/horseshoe_regression.py:33-49): unscaled_betas ~ Normal(0, 1)^P,
      beta = tau * lambdas * unscaled_betas (deterministic)
  StochasticVolatility (examples/stochastic_volatility.py:58-66)
      s ~ Exponential(s_rate); nu ~ Exponential(nu_rate)
      h ~ GaussianRandomWalk(scale=s, num_steps=T); r_t ~ StudentT(nu, 0, exp(h_t))
      noncentered=True: h_base ~ Normal(0, 1)^T; h = s * cumsum(h_base) (deterministic)
"""
from collections import namedtuple
import ctypes

import numpy as np

from . import _lib

Site = namedtuple("Site", ["name", "size", "positive"])



def _is_tensor(x):
    return hasattr(x, "detach") and hasattr(x, "device")


def _exp(v):
    return v.exp() if _is_tensor(v) else np.exp(v)

class Model:
    """Base class of registry models (the ``model=`` argument of NUTS/HMC)."""

    family = None
    sites = ()

    @property
    def latent_dim(self):
        return sum(s.size for s in self.sites)

    def chain_latent_dim(self, chain):
        return self.latent_dim

    def descriptor(self):
        """(ModelDesc, keepalive) for gbn_create."""
        raise NotImplementedError

    def site_slices(self):
        out, o = {}, 0
        for s in self.sites:
            out[s.name] = (o, o + s.size, s.positive)
            o += s.size
        return out

    def postprocess(self, z):
        """Unconstrained [..., D] -> dict of constrained site values (numpy arrays, or torch tensors
        on their own device when z is one: draws kept in HBM stay there)."""
        z = z if _is_tensor(z) else np.asarray(z)
        out = {}
        for name, (a, b, positive) in self.site_slices().items():
            v = z[..., a:b]
            out[name] = _exp(v) if positive else v
        return out

    def unravel(self, z):
        z = z if _is_tensor(z) else np.asarray(z)
        return {name: z[..., a:b] for name, (a, b, _) in self.site_slices().items()}


def _fp(a):
    return a.ctypes.data_as(_lib.c_float_p)


class HierarchicalNormal(Model):
    """One or many independent non-centred hierarchical-normal datasets.

    ``datasets`` is a list of (y_k, sigma_k) pairs of possibly different length
    J_k; chain c runs dataset c // chains_per_model.  With several datasets of
    uneven size, latent vectors are padded to max_k J_k + 2 (padding stays 0).
    """

    family = _lib.FAMILY_HIER_NC

    def __init__(self, y=None, sigma=None, datasets=None, mu_scale=5.0, tau_scale=5.0):
        if datasets is None:
            datasets = [(y, sigma)]
        self.datasets = [(np.asarray(a, np.float32).ravel(), np.asarray(b, np.float32).ravel()) for a, b in datasets]
        for a, b in self.datasets:
            if a.shape != b.shape:
                raise ValueError("y and sigma must have the same length")
        self.mu_scale = float(mu_scale)
        self.tau_scale = float(tau_scale)
        self.J = np.array([a.size for a, _ in self.datasets], np.int32)
        jmax = int(self.J.max())
        self.sites = (Site("mu", 1, False), Site("tau", 1, True), Site("theta_base", jmax, False))

    @property
    def num_models(self):
        return len(self.datasets)

    def chain_latent_dim(self, chain, chains_per_model=1):
        return int(self.J[chain // chains_per_model]) + 2

    def descriptor(self):
        y = np.ascontiguousarray(np.concatenate([a for a, _ in self.datasets]).astype(np.float32))
        s = np.ascontiguousarray(np.concatenate([b for _, b in self.datasets]).astype(np.float32))
        off = np.zeros(self.num_models + 1, np.int32)
        off[1:] = np.cumsum(self.J)
        d = _lib.ModelDesc()
        d.family = self.family
        d.num_models = self.num_models
        d.n = int(y.size)
        d.p = 0
        d.y = _fp(y)
        d.sigma = _fp(s)
        d.offsets = off.ctypes.data_as(_lib.c_int32_p)
        d.hyper[0] = self.mu_scale
        d.hyper[1] = self.tau_scale
        return d, (y, s, off)

    def postprocess(self, z):
        out = super().postprocess(z)
        out["theta"] = out["mu"] + out["tau"] * out["theta_base"]
        return out


class LogisticRegression(Model):
    family = _lib.FAMILY_LOGREG

    def __init__(self, X, y, prior_scale=1.0):
        self.X = np.ascontiguousarray(np.asarray(X, np.float32))
        self.y = np.ascontiguousarray(np.asarray(y, np.float32).ravel())
        if self.X.ndim != 2 or self.X.shape[0] != self.y.shape[0]:
            raise ValueError("X must be [N, D] and y [N]")
        self.prior_scale = float(prior_scale)
        self.sites = (Site("coefs", self.X.shape[1], False),)

    def descriptor(self):
        d = _lib.ModelDesc()
        d.family = self.family
        d.num_models = 1
        d.n = self.X.shape[0]
        d.p = self.X.shape[1]
        d.x = _fp(self.X)
        d.y = _fp(self.y)
        d.hyper[0] = self.prior_scale
        return d, (self.X, self.y)


class HorseshoeRegression(Model):
    family = _lib.FAMILY_HORSESHOE

    def __init__(self, X, y, noncentered=False):
        self.X = np.ascontiguousarray(np.asarray(X, np.float32))
        self.y = np.ascontiguousarray(np.asarray(y, np.float32).ravel())
        self.noncentered = bool(noncentered)
        P = self.X.shape[1]
        if self.noncentered:
            self.sites = (Site("lambdas", P, True), Site("sigma", 1, True), Site("tau", 1, True),
                          Site("unscaled_betas", P, False))
        else:
            self.sites = (Site("beta", P, False), Site("lambdas", P, True), Site("sigma", 1, True),
                          Site("tau", 1, True))

    def postprocess(self, z):
        out = super().postprocess(z)
        if self.noncentered:
            out["beta"] = out["tau"] * out["lambdas"] * out["unscaled_betas"]
        return out

    def descriptor(self):
        d = _lib.ModelDesc()
        d.family = self.family
        d.num_models = 1
        d.n = self.X.shape[0]
        d.p = self.X.shape[1]
        d.x = _fp(self.X)
        d.y = _fp(self.y)
        d.hyper[0] = 1.0 if self.noncentered else 0.0
        return d, (self.X, self.y)


class StochasticVolatility(Model):
    family = _lib.FAMILY_SV

    def __init__(self, returns, s_rate=10.0, nu_rate=0.1, noncentered=False):
        self.returns = np.ascontiguousarray(np.asarray(returns, np.float32).ravel())
        self.s_rate = float(s_rate)
        self.nu_rate = float(nu_rate)
        self.noncentered = bool(noncentered)
        T = self.returns.size
        walk = "h_base" if self.noncentered else "h"
        self.sites = (Site(walk, T, False), Site("nu", 1, True), Site("s", 1, True))

    def postprocess(self, z):
        out = super().postprocess(z)
        if self.noncentered:
            hb = out["h_base"]
            out["h"] = out["s"] * (hb.cumsum(dim=-1) if _is_tensor(hb) else np.cumsum(hb, axis=-1))
        return out

    def descriptor(self):
        d = _lib.ModelDesc()
        d.family = self.family
        d.num_models = 1
        d.n = self.returns.size
        d.y = _fp(self.returns)
        d.hyper[0] = self.s_rate
        d.hyper[1] = self.nu_rate
        d.hyper[2] = 1.0 if self.noncentered else 0.0
        return d, (self.returns,)


REGISTRY = {
    "hier_nc": HierarchicalNormal,
    "logreg": LogisticRegression,
    "horseshoe": HorseshoeRegression,
    "sv": StochasticVolatility,
}
