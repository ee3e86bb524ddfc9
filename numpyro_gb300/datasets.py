"""Seeded synthetic datasets with the shapes of the benchmark workloads.

The reference's own hot-path examples load covtype and SP500 over the network
(numpyro/examples/datasets.py:289-292, :345-349); those are unavailable, so
these generators stand in for them with the same shapes and value
distributions.  Every generator is deterministic in its seed.
"""
import numpy as np


def _round_bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def eight_schools(seed=0, J=8):
    """J groups: sigma_j ~ U(9, 18); mu = 4, tau = 3; theta_j ~ N(mu, tau); y_j ~ N(theta_j, sigma_j)."""
    rng = np.random.default_rng(seed)
    sigma = rng.uniform(9.0, 18.0, J)
    theta = 4.0 + 3.0 * rng.standard_normal(J)
    y = theta + sigma * rng.standard_normal(J)
    return y.astype(np.float32), sigma.astype(np.float32)


def covtype_like(seed=0, n=581012, n_cont=10, n_bin=44, bf16_exact=True):
    """covtype-shaped logistic-regression data (examples/covtype.py:43-71).

    10 continuous N(0,1) columns (rounded to bfloat16 when ``bf16_exact`` so
    that the tensor-core path sees exactly the data the FP32/FP64 paths see),
    44 Bernoulli(0.05) columns and an intercept column of ones; true
    coefficients ~ N(0,1)/sqrt(55); y ~ Bernoulli(sigmoid(X beta*)).
    """
    rng = np.random.default_rng(seed)
    d = n_cont + n_bin + 1
    X = np.empty((n, d), np.float32)
    cont = rng.standard_normal((n, n_cont)).astype(np.float32)
    X[:, :n_cont] = _round_bf16(cont) if bf16_exact else cont
    X[:, n_cont:n_cont + n_bin] = (rng.random((n, n_bin)) < 0.05).astype(np.float32)
    X[:, -1] = 1.0
    beta = rng.standard_normal(d) / np.sqrt(d)
    logits = X.astype(np.float64) @ beta
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-logits))).astype(np.float32)
    return X, y, beta


def uneven_hierarchical(seed=0, num_models=4096, jmin=4, jmax=256):
    """num_models datasets: J_k ~ UniformInt[jmin, jmax], sigma ~ U(1, 20),
    mu_k ~ N(0, 5), tau_k ~ HalfCauchy(3), y from the model."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(num_models):
        J = int(rng.integers(jmin, jmax + 1))
        sigma = rng.uniform(1.0, 20.0, J)
        mu = 5.0 * rng.standard_normal()
        tau = abs(3.0 * rng.standard_cauchy())
        theta = mu + tau * rng.standard_normal(J)
        y = theta + sigma * rng.standard_normal(J)
        out.append((y.astype(np.float32), sigma.astype(np.float32)))
    return out


def horseshoe_data(seed=0, n=2000, p=1000, nonzero=10, rho=0.5):
    """Rows ~ N(0, Sigma), Sigma_ij = rho^|i-j| (AR(1) recursion); 10 nonzero
    coefficients +-U(1,3) at random indices; y = X beta + N(0, 1)."""
    rng = np.random.default_rng(seed)
    e = rng.standard_normal((n, p))
    X = np.empty((n, p))
    X[:, 0] = e[:, 0]
    c = np.sqrt(1.0 - rho * rho)
    for j in range(1, p):
        X[:, j] = rho * X[:, j - 1] + c * e[:, j]
    beta = np.zeros(p)
    idx = rng.choice(p, nonzero, replace=False)
    beta[idx] = rng.choice([-1.0, 1.0], nonzero) * rng.uniform(1.0, 3.0, nonzero)
    y = X @ beta + rng.standard_normal(n)
    return X.astype(np.float32), y.astype(np.float32), beta


def sv_returns(seed=0, T=4096, s=0.02, nu=8.0, h0=np.log(0.01)):
    """h_t = h_{t-1} + s eps_t from h_0 = log 0.01; r_t ~ StudentT(nu, 0, exp(h_t))."""
    rng = np.random.default_rng(seed)
    h = h0 + np.cumsum(s * rng.standard_normal(T))
    r = np.exp(h) * rng.standard_t(nu, T)
    return r.astype(np.float32), h
