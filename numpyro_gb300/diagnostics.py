# Portions of this file (the estimators from _compute_chain_variance_stats to
# effective_sample_size) are adapted from numpyro/diagnostics.py of NumPyro,
# Copyright Contributors to the Pyro project, licensed under the Apache License,
# Version 2.0 (http://www.apache.org/licenses/LICENSE-2.0).  They are kept
# statement-for-statement equivalent on purpose: the R-hat gate and the ESS known
# answers of the benchmark are numpyro's own.
"""MCMC diagnostics (numpyro/diagnostics.py restated, plus rank-normalised bulk ESS).

``effective_sample_size``, ``split_gelman_rubin``, ``gelman_rubin``,
``autocorrelation``, ``autocovariance``, ``hpdi``, ``summary`` and
``print_summary`` follow numpyro/diagnostics.py:29-345 (the benchmark's R-hat
gate uses split_gelman_rubin, :64-80).  ``bulk_effective_sample_size`` is the
rank-normalised split-ESS of Vehtari, Gelman, Simpson, Carpenter and Buerkner
(2021), the "bulk-ESS" of the benchmark metric.
"""
import numpy as np
from scipy.special import ndtri


def _compute_chain_variance_stats(x):
    """diagnostics.py:29-42"""
    C, N = x.shape[:2]
    chain_var = x.var(axis=1, ddof=1)
    var_within = chain_var.mean(axis=0)
    var_estimator = var_within * (N - 1) / N
    if x.shape[0] > 1:
        chain_mean = x.mean(axis=1)
        var_between = chain_mean.var(axis=0, ddof=1)
        var_estimator = var_estimator + var_between
    else:
        var_within = var_estimator
    return var_within, var_estimator


def gelman_rubin(x):
    """diagnostics.py:45-61"""
    assert x.ndim >= 2 and x.shape[0] >= 2 and x.shape[1] >= 2
    var_within, var_estimator = _compute_chain_variance_stats(x)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.sqrt(var_estimator / var_within)


def split_gelman_rubin(x):
    """diagnostics.py:64-80"""
    assert x.ndim >= 2 and x.shape[1] >= 4
    n_half = x.shape[1] // 2
    return gelman_rubin(np.concatenate([x[:, :n_half], x[:, -n_half:]], axis=0))


def _fft_next_fast_len(target):
    """diagnostics.py:83-98"""
    if target <= 2:
        return target
    while True:
        m = target
        while m % 2 == 0:
            m //= 2
        while m % 3 == 0:
            m //= 3
        while m % 5 == 0:
            m //= 5
        if m == 1:
            return target
        target += 1


def autocorrelation(x, axis=0, bias=True):
    """diagnostics.py:101-142"""
    N = x.shape[axis]
    M2 = 2 * _fft_next_fast_len(N)
    x = np.swapaxes(x, axis, -1)
    centered = x - x.mean(axis=-1, keepdims=True)
    freq = np.fft.rfft(centered, n=M2, axis=-1)
    ac = np.fft.irfft(freq * np.conjugate(freq), n=M2, axis=-1)[..., :N]
    if not bias:
        ac = ac / np.arange(N, 0.0, -1)
    with np.errstate(invalid="ignore", divide="ignore"):
        ac = (ac / ac[..., :1]).astype(np.float64)
    return np.swapaxes(ac, axis, -1)


def autocovariance(x, axis=0, bias=True):
    """diagnostics.py:145-155"""
    return autocorrelation(x, axis, bias) * x.var(axis=axis, keepdims=True)


def effective_sample_size(x, bias=True):
    """diagnostics.py:158-203 (Geyer initial positive + monotone sequence)."""
    x = np.asarray(x, np.float64)
    assert x.ndim >= 2 and x.shape[1] >= 2
    gamma_k_c = autocovariance(x, axis=1, bias=bias)
    var_within, var_estimator = _compute_chain_variance_stats(x)
    rho_k = 1.0 - (var_within - gamma_k_c.mean(axis=0)) / var_estimator
    rho_k[0] = 1.0
    Rho_k = rho_k[:-1:2, ...] + rho_k[1::2, ...]
    Rho_init = Rho_k[:1]
    Rho_k = np.concatenate([Rho_init, np.minimum.accumulate(np.clip(Rho_k[1:, ...], 0, None), axis=0)], axis=0)
    tau = -1.0 + 2.0 * Rho_k.sum(axis=0)
    return np.prod(x.shape[:2]) / tau


def mcse_mean(x):
    """Monte Carlo standard error of the posterior mean of each coordinate of x [C, S, ...]:
    sd / sqrt(ESS), with numpyro's effective_sample_size."""
    x = np.asarray(x, np.float64)
    sd = x.reshape((-1,) + x.shape[2:]).std(axis=0, ddof=1)
    return sd / np.sqrt(effective_sample_size(x))


def mcse_sd(x):
    """Monte Carlo standard error of the posterior sd of each coordinate of x [C, S, ...]: the
    delta method on the variance, whose own error is that of the mean of the squared deviations
    (their ESS, not the draws' -- NUTS draws are often antithetic for x but not for x^2):
    mcse(sd) = sqrt(var(d^2) / ESS(d^2)) / (2 sd), d = x - mean (Vehtari et al. 2021, sec. 3)."""
    x = np.asarray(x, np.float64)
    flat = x.reshape((-1,) + x.shape[2:])
    m = flat.mean(axis=0)
    sd = flat.std(axis=0, ddof=1)
    d2 = (x - m) ** 2
    var_d2 = d2.reshape((-1,) + x.shape[2:]).var(axis=0, ddof=1)
    return np.sqrt(var_d2 / effective_sample_size(d2)) / (2.0 * sd)


def _split_chains(x):
    n_half = x.shape[1] // 2
    return np.concatenate([x[:, :n_half], x[:, -n_half:]], axis=0)


def rank_normalize(x):
    """z-scores of pooled fractional ranks, (r - 3/8) / (S - 1/4) (Vehtari et al. 2021, eq. 14)."""
    from scipy.stats import rankdata

    shp = x.shape
    flat = x.reshape(shp[0] * shp[1], -1)
    r = rankdata(flat, axis=0, method="average")
    z = ndtri((r - 0.375) / (flat.shape[0] + 0.25))
    return z.reshape(shp)


def bulk_effective_sample_size(x):
    """Rank-normalised split-chain ESS ("bulk-ESS", Vehtari et al. 2021).

    The autocorrelation sum follows effective_sample_size (Geyer's initial
    monotone sequence); as in Vehtari et al. the integrated autocorrelation
    time is bounded below by 1/log10(total draws), which keeps antithetic
    (negatively autocorrelated) NUTS draws from short chains finite and
    positive."""
    z = rank_normalize(_split_chains(np.asarray(x, np.float64)))
    total = np.prod(z.shape[:2])
    ess = effective_sample_size(z)
    tau = total / ess
    floor = 1.0 / np.log10(total)
    # a non-positive Geyer sum means antithetic draws beyond what the chains can resolve
    tau = np.where(np.isfinite(tau) & (tau > 0), np.maximum(tau, floor), floor)
    return total / tau


def rank_split_rhat(x):
    x = np.asarray(x, np.float64)
    return gelman_rubin(rank_normalize(_split_chains(x)))


def hpdi(x, prob=0.90, axis=0):
    """diagnostics.py:206-232"""
    x = np.swapaxes(x, axis, 0)
    sorted_x = np.sort(x, axis=0)
    mass = x.shape[0]
    index_length = int(prob * mass)
    intervals_left = sorted_x[: (mass - index_length)]
    intervals_right = sorted_x[index_length:]
    intervals_length = intervals_right - intervals_left
    index_start = intervals_length.argmin(axis=0)
    index_end = index_start + index_length
    hpd_left = np.take_along_axis(sorted_x, index_start[None, ...], axis=0)
    hpd_right = np.take_along_axis(sorted_x, index_end[None, ...], axis=0)
    return np.swapaxes(np.concatenate([hpd_left, hpd_right], axis=0), axis, 0)


def summary(samples, prob=0.90, group_by_chain=True):
    """diagnostics.py:235-287: dict site -> stats (mean, std, median, hpdi, n_eff, r_hat)."""
    if not isinstance(samples, dict):
        samples = {"Param:{}".format(i): v for i, v in enumerate(samples)}
    if not group_by_chain:
        samples = {k: v[None, ...] for k, v in samples.items()}
    out = {}
    for name, value in samples.items():
        value = np.asarray(value)
        value_flat = value.reshape((-1,) + value.shape[2:])
        mean = value_flat.mean(axis=0)
        std = value_flat.std(axis=0, ddof=1)
        median = np.median(value_flat, axis=0)
        hpd = hpdi(value_flat, prob=prob)
        n_eff = effective_sample_size(value)
        r_hat = split_gelman_rubin(value)
        lo, hi = 50 * (1 - prob), 50 * (1 + prob)
        out[name] = {"mean": mean, "std": std, "median": median, "{:.1f}%".format(lo): hpd[0],
                     "{:.1f}%".format(hi): hpd[1], "n_eff": n_eff, "r_hat": r_hat}
    return out


def print_summary(samples, prob=0.90, group_by_chain=True):
    """diagnostics.py:290-345"""
    print_stats(summary(samples, prob, group_by_chain))


def print_stats(stats):
    """The table of print_summary from summary()'s dict (also fed by device_diagnostics.summary)."""
    if not stats:
        return
    first = next(iter(stats.values()))
    cols = list(first.keys())
    print("{:>20}".format("") + "".join("{:>10}".format(c) for c in cols))
    for name, s in stats.items():
        shape = np.shape(s["mean"])
        if len(shape) == 0:
            print("{:>20}".format(name) + "".join("{:>10.2f}".format(float(s[c])) for c in cols))
        else:
            for idx in np.ndindex(shape):
                label = "{}[{}]".format(name, ",".join(map(str, idx)))
                print("{:>20}".format(label) + "".join("{:>10.2f}".format(float(s[c][idx])) for c in cols))
    print()
