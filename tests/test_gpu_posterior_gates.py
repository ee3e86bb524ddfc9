"""Posterior gates at reduced sizes of the benchmark configurations, against the FP64 oracle.

The benchmark's correctness criterion: split R-hat (numpyro/diagnostics.py:64-80) < 1.01 for
every coordinate, and the posterior means and sds within 3 Monte Carlo standard errors of the
FP64 oracle's (the Monte Carlo standard errors of both samples combined in quadrature:
numpyro_gb300.diagnostics.mcse_mean and mcse_sd, the latter from the ESS of the squared
deviations).  With n comparisons (two per coordinate, up to ~1,000 here) a correct sampler puts
about 0.27 % of them beyond 3 MCSE by chance alone (some with probability 1 - 0.9973^n: 26 % for
n = 110, 94 % for n = 1,028), so the gate asks what chance allows: at most n p3 + 3 sqrt(n p3) + 1
comparisons beyond 3 MCSE (p3 = 0.0027), and every one within the Bonferroni bound
Phi^-1(1 - 0.005 / n) (3.9 for n = 110, 4.4 for n = 1,028).  The oracle is the FP64 C restatement
of numpyro's NUTS (oracle/nuts_ref.c), run on the host cores: with its own Stan warmup from
init_to_uniform where that is cheap, or, for the logistic model, from the GPU's adapted state (its
first draws are discarded, so a GPU posterior that were off would show as the oracle chains
drifting away from it).  The horseshoe gate calibrates its MCSEs by two oracle runs (see there).

Sizes: logistic 20,000 rows x 55 coefficients (FP32 CUDA cores and bf16x3 tensor cores),
stochastic volatility T = 512, non-centred horseshoe N = 200, P = 50 (FP32 and bf16x3), and
8 uneven hierarchical datasets (J from 4 to 64) in one launch.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import NUTS, datasets, models  # noqa: E402
from numpyro_gb300.diagnostics import (bulk_effective_sample_size, mcse_mean, mcse_sd,  # noqa: E402
                                       split_gelman_rubin)
from oracle import build_oracle as B  # noqa: E402

from gpu_helpers import cmodel_of  # noqa: E402

SEED = 11


def _stats(z):
    z = np.asarray(z, np.float64)
    m = z.mean(axis=(0, 1))
    sd = z.std(axis=(0, 1), ddof=1)
    ess = np.atleast_1d(bulk_effective_sample_size(z))
    rhat = np.atleast_1d(split_gelman_rubin(z))
    return m, sd, mcse_mean(z), mcse_sd(z), ess, rhat


def moment_bounds(n):
    """For n comparisons of independent estimates in units of their MCSE: the most that may lie
    beyond 3 MCSE by chance (binomial mean + 3 sd, plus one) and the bound every one must meet
    (Bonferroni at a family-wise false-alarm rate of 1 %: Phi^-1(1 - 0.005 / n))."""
    from scipy.stats import norm

    p3 = 2 * norm.sf(3.0)
    return int(np.floor(n * p3 + 3 * np.sqrt(n * p3 * (1 - p3)) + 1)), float(norm.isf(0.005 / n))


def _z(zg, zo, conv_rhat):
    """|difference| / combined MCSE of each coordinate's mean and sd between two samples, on the
    coordinates both have mixed on; with the statistics."""
    mg, sg, emg, esg, eg, rg = _stats(zg)
    mo, so, emo, eso, eo, ro = _stats(zo)
    conv = (rg < conv_rhat) & (ro < conv_rhat)
    zm = (np.abs(mg - mo) / np.sqrt(emg ** 2 + emo ** 2))[conv]
    zs = (np.abs(sg - so) / np.sqrt(esg ** 2 + eso ** 2))[conv]
    return zm, zs, conv, (mg, sg, eg, rg), (mo, so, eo, ro)


def mcse_inflation(za, zb, conv_rhat):
    """How far two runs of the reference sampler part in units of their own combined MCSEs:
    sqrt(mean z^2) over the means and sds of the coordinates both mixed on (1 if the MCSEs are
    right; never below 1)."""
    zm, zs, _, _, _ = _z(za, zb, conv_rhat)
    return max(1.0, float(np.sqrt(np.mean(np.concatenate([zm, zs]) ** 2))))


def _gate(name, zg, zo, rhat_max=1.01, max_unconverged=0.0, conv_rhat=1.01, inflation=1.0):
    """R-hat of the GPU chains below rhat_max; the moments of every coordinate that both samples
    have mixed on (split R-hat < conv_rhat: a Monte Carlo standard error means nothing otherwise)
    within what chance allows, in units of the combined MCSE times `inflation`; at most
    max_unconverged of the coordinates left out."""
    zm, zs, conv, (mg, sg, eg, rg), (mo, so, eo, ro) = _z(zg, zo, conv_rhat)
    zm, zs = zm / inflation, zs / inflation
    z = np.concatenate([zm, zs])
    beyond3, bound = moment_bounds(z.size)
    print("%s: GPU R-hat max %.4f (oracle %.4f), min bulk-ESS GPU %.0f oracle %.0f; "
          "max |dmean|/MCSE %.2f, max |dsd|/MCSE %.2f over %d mixed coordinates (of %d); %d of %d comparisons "
          "beyond 3 MCSE (chance allows %d), all within %.2f"
          % (name, rg.max(), ro.max(), eg.min(), eo.min(), zm.max(), zs.max(), zm.size, conv.size, np.sum(z > 3),
             z.size, beyond3, bound))
    idx = np.flatnonzero(conv)
    for j in np.flatnonzero(z > 3.0):
        kind, i = ("mean", idx[j]) if j < zm.size else ("sd", idx[j - zm.size])
        a, b = (mg[i], mo[i]) if kind == "mean" else (sg[i], so[i])
        print("  beyond 3 MCSE: coordinate %d %s %.5f (GPU) vs %.5f (oracle), z = %.2f" % (i, kind, a, b, z[j]))
    assert np.mean(~conv) <= max_unconverged, (name, int(np.sum(~conv)))
    assert rg.max() < rhat_max, (name, rg.max())
    assert np.sum(z > 3.0) <= beyond3, (name, int(np.sum(z > 3.0)))
    coord = np.flatnonzero(conv)[int(np.argmax(z)) % zm.size]
    assert z.max() <= bound, (name, "mean" if np.argmax(z) < zm.size else "sd", int(coord), z.max())


def _gpu_run(model, C, W, S, with_divergences=False, **kw):
    k = NUTS(model, num_chains=C, **kw)
    st = k.init(SEED, W)
    k.run_device(st, W, collect_start=W, collect=())
    out = k.run_device(st, S, collect=("z", "diverging"))
    z = out["z"].cpu().numpy()
    div = out["diverging"].cpu().numpy()
    k.close()
    return (z, st, div) if with_divergences else (z, st)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_logistic_posterior_gate(precision):
    X, y, _ = datasets.covtype_like(seed=5, n=20_000)
    model = models.LogisticRegression(X, y)
    zg, st = _gpu_run(model, 256, 300, 300, precision=precision)
    nc = 16
    init = (st.z[:nc].cpu().numpy(), st.adapt_state.step_size[:nc].cpu().numpy(),
            st.adapt_state.inverse_mass_matrix[:nc].cpu().numpy())
    res = B.run_model(B.load("f64"), cmodel_of(model), X.shape[1], nc, 0, 350, seed=SEED + 1, init=init)
    _gate("logistic N=20000 %s" % precision, zg, res["samples"][:, 50:])


@pytest.mark.gpu
def test_stochastic_volatility_posterior_gate():
    r, _ = datasets.sv_returns(seed=0, T=512)
    model = models.StochasticVolatility(r)
    # 1000 + 1000 leaves both the GPU (R-hat 1.019 over 64 chains) and numpyro's algorithm (1.021 over
    # 16 chains) short of R-hat 1.01 on this posterior (s and nu mix slowly); 3000 draws reach it
    zg, _ = _gpu_run(model, 64, 1000, 3000)
    res = B.run_model(B.load("f64"), cmodel_of(model), model.latent_dim, 16, 1000, 3000, seed=SEED + 2)
    _gate("sv T=512", zg, res["samples"])


# numpyro's algorithm itself does not reach split R-hat 1.01 on this horseshoe posterior: the FP64
# restatement with 128 chains, 1000 warmup + 3000 draws, ended at 1.010, 1.024, 1.083 and 1.116 over
# four seeds (6.9-9.3 % of its transitions divergent; the half-Cauchy local scales of the null
# coefficients leave funnels that some chains cross rarely).  So the GPU's R-hat is held to the
# reference sampler's own range on the same posterior, chains and draws, and its divergence rate to
# within half and one and a half times the oracle's.  The moments are compared on the coordinates
# whose split R-hat is below 1.05 in both samples (at most a quarter may be left out).  On this
# posterior the Monte Carlo standard errors understate how far runs part: three oracle runs put one
# coefficient's sd at 0.846 (16 chains), 0.859 and 0.871 (64 chains each), with MCSEs of 0.005-0.006.
# So two oracle runs of 64 chains (different seeds) measure that understatement -- sqrt(mean z^2) of
# their own moments in units of their combined MCSEs -- and the GPU is compared with the two pooled
# in units inflated by it.
HORSESHOE_RHAT_OF_REFERENCE = 1.12


@pytest.fixture(scope="module")
def horseshoe_oracle():
    X, y, _ = datasets.horseshoe_data(seed=3, n=200, p=50, nonzero=5)
    model = models.HorseshoeRegression(X, y, noncentered=True)
    lib = B.load("f64")
    runs = [B.run_model(lib, cmodel_of(model), model.latent_dim, 64, 1000, 3000, seed=SEED + 3 + 100 * r,
                        first_chain=64 * r) for r in range(2)]
    return model, runs


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_horseshoe_posterior_gate(precision, horseshoe_oracle):
    model, runs = horseshoe_oracle
    kappa = mcse_inflation(runs[0]["samples"], runs[1]["samples"], 1.05)
    zo = np.concatenate([r["samples"] for r in runs], axis=0)
    print("two oracle runs part by %.2f of their combined MCSEs (rms over means and sds)" % kappa)
    zg, _, dg = _gpu_run(model, 128, 1000, 3000, with_divergences=True, precision=precision)
    _gate("horseshoe_nc N=200 P=50 %s" % precision, zg, zo, rhat_max=HORSESHOE_RHAT_OF_REFERENCE,
          max_unconverged=0.25, conv_rhat=1.05, inflation=kappa)
    fg, fo = dg.mean(), np.concatenate([r["diverging"] for r in runs]).mean()
    print("divergent transitions: GPU %.4f, oracle %.4f" % (fg, fo))
    assert 0.5 * fo <= fg <= 1.5 * fo, (fg, fo)


@pytest.mark.gpu
def test_uneven_hierarchical_posterior_gate():
    ds = datasets.uneven_hierarchical(seed=4, num_models=8, jmin=4, jmax=64)
    model = models.HierarchicalNormal(datasets=ds)
    cpm = 16
    zg, _ = _gpu_run(model, cpm * len(ds), 1000, 1000)
    cm = cmodel_of(model, chains_per_model=cpm)
    lib = B.load("f64")
    for k, (yk, _) in enumerate(ds):
        D = len(yk) + 2
        # the oracle's chains of dataset k: global chain ids k * cpm .. k * cpm + 7
        res = B.run_model(lib, cm, model.latent_dim, 8, 1000, 1000, seed=SEED + 4, first_chain=k * cpm)
        _gate("uneven hierarchical dataset %d (J=%d)" % (k, len(yk)), zg[k * cpm:(k + 1) * cpm, :, :D],
              res["samples"][:, :, :D])
