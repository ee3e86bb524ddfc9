"""Shared helpers for the GPU parity tests (imports the oracle as the checker)."""
import numpy as np

from numpyro_gb300 import datasets, models
from oracle import potentials_ref as PR


def family_cases(small=True):
    """(name, registry model, oracle potential_and_grad) for each family at test sizes."""
    out = []
    y, s = datasets.eight_schools(0)
    out.append(("hier_nc", models.HierarchicalNormal(y, s), PR.make_potential("hier_nc", y.astype(np.float64),
                                                                                s.astype(np.float64))))
    X, yy, _ = datasets.covtype_like(seed=1, n=3000 if small else 581012, n_cont=4, n_bin=6)
    out.append(("logreg", models.LogisticRegression(X, yy), PR.make_potential("logreg", X.astype(np.float64),
                                                                              yy.astype(np.float64))))
    Xh, yh, _ = datasets.horseshoe_data(seed=2, n=200, p=50, nonzero=5)
    out.append(("horseshoe", models.HorseshoeRegression(Xh, yh),
                PR.make_potential("horseshoe", Xh.astype(np.float64), yh.astype(np.float64))))
    out.append(("horseshoe_nc", models.HorseshoeRegression(Xh, yh, noncentered=True),
                PR.make_potential("horseshoe_nc", Xh.astype(np.float64), yh.astype(np.float64))))
    r, _ = datasets.sv_returns(seed=3, T=300)
    out.append(("sv", models.StochasticVolatility(r), PR.make_potential("sv", r.astype(np.float64))))
    r2, _ = datasets.sv_returns(seed=4, T=1000)
    out.append(("sv_nc", models.StochasticVolatility(r2, noncentered=True),
                PR.make_potential("sv_nc", r2.astype(np.float64))))
    return out


def typical_points(name, model, rng, C):
    """Latent points in a plausible region of each posterior."""
    D = model.latent_dim
    if name == "sv":
        T = D - 2
        z = np.empty((C, D))
        z[:, :T] = np.log(0.01) + 0.3 * rng.standard_normal((C, T))
        z[:, T] = np.log(8.0) + 0.3 * rng.standard_normal(C)
        z[:, T + 1] = np.log(0.02) + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    if name == "sv_nc":
        T = D - 2
        z = np.empty((C, D))
        z[:, :T] = 0.3 * rng.standard_normal((C, T))
        z[:, T] = np.log(8.0) + 0.3 * rng.standard_normal(C)
        z[:, T + 1] = np.log(0.05) + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    if name == "logreg":
        return (0.3 * rng.standard_normal((C, D))).astype(np.float32)
    if name == "horseshoe_nc":
        P = (D - 2) // 2
        z = np.empty((C, D))
        z[:, :P] = rng.standard_normal((C, P))
        z[:, P] = 0.3 * rng.standard_normal(C)
        z[:, P + 1] = -2.0 + 0.3 * rng.standard_normal(C)
        z[:, P + 2:] = rng.standard_normal((C, P))
        return z.astype(np.float32)
    if name == "horseshoe":
        P = (D - 2) // 2
        z = np.empty((C, D))
        z[:, :P] = 0.1 * rng.standard_normal((C, P))
        z[:, P:2 * P] = rng.standard_normal((C, P))
        z[:, 2 * P] = 0.3 * rng.standard_normal(C)
        z[:, 2 * P + 1] = -2.0 + 0.3 * rng.standard_normal(C)
        return z.astype(np.float32)
    return rng.uniform(-2, 2, (C, D)).astype(np.float32)
