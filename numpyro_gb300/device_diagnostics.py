"""MCMC diagnostics on the device: the estimators of ``numpyro_gb300.diagnostics`` (numpyro's split
R-hat and Geyer ESS, numpyro/diagnostics.py:29-203; rank-normalised bulk-ESS, Vehtari et al. 2021)
for draws that stay in HBM.

numpyro computes these on the host after ``fori_collect`` has copied every draw back
(numpyro/infer/mcmc.py:687-724, diagnostics.py:235-287).  At the benchmark's sizes the draws are
gigabytes (256 chains x 1000 draws x 4,098 coordinates for the stochastic-volatility model), so
here the statistics are formed where the draws are, and only the per-coordinate results move.
Every function takes a torch tensor ``x`` of shape [chains, draws, ...] on any device, computes in
float64 by default, and walks the trailing coordinates in chunks (``chunk`` coordinates at a time)
so that the FFT and sort buffers stay bounded.  The results equal the host versions to rounding
(tests/test_diagnostics_cpu.py compares them on CPU tensors, tests/test_gpu_mcmc.py on the GPU).

Ties: a rejected NUTS transition repeats its draw, so equal values are common; ranks are averaged
over ties (scipy.stats.rankdata's "average"), as the host version does.
"""
import math

import torch

__all__ = ["split_gelman_rubin", "gelman_rubin", "effective_sample_size", "rank_normalize",
           "bulk_effective_sample_size", "mcse_mean", "mcse_sd", "summary_stats", "hpdi", "summary"]


def _blocks(x, chunk, dtype):
    """Yields blocks [C, S, k] in dtype of x [C, S, ...], about `chunk` coordinates per block, split
    along the first trailing dimension; only a block is ever converted or copied, so x may be a
    large non-contiguous view (the chains of each model as the leading dimension, for instance)."""
    if not torch.is_tensor(x):
        raise TypeError("device diagnostics take a torch tensor [chains, draws, ...]")
    if x.dim() < 2:
        raise ValueError("x must be [chains, draws, ...]")
    if x.dim() == 2:
        x = x.unsqueeze(-1)
    C, S, lead = x.shape[:3]
    inner = 1
    for n in x.shape[3:]:
        inner *= n
    step = max(1, chunk // max(inner, 1))
    for a in range(0, lead, step):
        yield x[:, :, a:a + step].reshape(C, S, -1).to(dtype)


def _chain_variance_stats(x):
    """diagnostics.py:29-42 for x [C, N, K]."""
    C, N = x.shape[:2]
    var_within = x.var(dim=1, unbiased=True).mean(dim=0)
    var_estimator = var_within * (N - 1) / N
    if C > 1:
        var_estimator = var_estimator + x.mean(dim=1).var(dim=0, unbiased=True)
    else:
        var_within = var_estimator
    return var_within, var_estimator


def _gelman_rubin(x):
    var_within, var_estimator = _chain_variance_stats(x)
    return torch.sqrt(var_estimator / var_within)


def _split(x):
    n_half = x.shape[1] // 2
    return torch.cat([x[:, :n_half], x[:, x.shape[1] - n_half:]], dim=0)


def _next_fast_len(target):
    """diagnostics.py:83-98"""
    if target <= 2:
        return target
    while True:
        m = target
        for f in (2, 3, 5):
            while m % f == 0:
                m //= f
        if m == 1:
            return target
        target += 1


def _autocovariance(x):
    """autocovariance along dim 1 of x [C, N, K] (diagnostics.py:101-155, bias=True)."""
    N = x.shape[1]
    M2 = 2 * _next_fast_len(N)
    centered = x - x.mean(dim=1, keepdim=True)
    freq = torch.fft.rfft(centered, n=M2, dim=1)
    ac = torch.fft.irfft(freq * freq.conj(), n=M2, dim=1)[:, :N]
    ac = ac / ac[:, :1]
    return ac * x.var(dim=1, unbiased=False, keepdim=True)


def _ess(x):
    """diagnostics.py:158-203 (Geyer initial positive + monotone sequence) for x [C, N, K]."""
    gamma = _autocovariance(x)
    var_within, var_estimator = _chain_variance_stats(x)
    rho = 1.0 - (var_within - gamma.mean(dim=0)) / var_estimator
    rho[0] = 1.0
    n_even = rho.shape[0] // 2
    Rho = rho[0:2 * n_even:2] + rho[1:2 * n_even:2]
    rest = torch.clamp(Rho[1:], min=0.0)
    if rest.shape[0] > 0:
        rest = torch.cummin(rest, dim=0).values
    Rho = torch.cat([Rho[:1], rest], dim=0)
    tau = -1.0 + 2.0 * Rho.sum(dim=0)
    return x.shape[0] * x.shape[1] / tau


def _rank_normalize(x):
    """z-scores of pooled average ranks, (r - 3/8) / (S - 1/4), for x [C, N, K]."""
    C, N, K = x.shape
    flat = x.reshape(C * N, K)
    S = flat.shape[0]
    v, order = torch.sort(flat, dim=0)
    idx = torch.arange(S, device=x.device).unsqueeze(1).expand(S, K)
    new_run = torch.ones_like(v, dtype=torch.bool)
    new_run[1:] = v[1:] != v[:-1]
    end_run = torch.ones_like(v, dtype=torch.bool)
    end_run[:-1] = v[:-1] != v[1:]
    first = torch.cummax(torch.where(new_run, idx, torch.zeros_like(idx)), dim=0).values
    last = torch.flip(torch.cummin(torch.flip(torch.where(end_run, idx, torch.full_like(idx, S - 1)), [0]),
                                   dim=0).values, [0])
    r_sorted = (first + last).to(x.dtype) * 0.5 + 1.0
    r = torch.empty_like(r_sorted)
    r.scatter_(0, order, r_sorted)
    z = torch.special.ndtri((r - 0.375) / (S + 0.25))
    return z.reshape(C, N, K)


def _apply(x, fn, chunk, dtype):
    return torch.cat([fn(t) for t in _blocks(x, chunk, dtype)]).reshape(tuple(x.shape[2:]))


def gelman_rubin(x, chunk=1024, dtype=torch.float64):
    """diagnostics.py:45-61 on the device."""
    if x.shape[0] < 2 or x.shape[1] < 2:
        raise ValueError("gelman_rubin needs at least 2 chains and 2 draws")
    return _apply(x, _gelman_rubin, chunk, dtype)


def split_gelman_rubin(x, chunk=1024, dtype=torch.float64):
    """diagnostics.py:64-80 on the device: the benchmark's R-hat gate."""
    if x.shape[1] < 4:
        raise ValueError("split_gelman_rubin needs at least 4 draws")
    return _apply(x, lambda t: _gelman_rubin(_split(t)), chunk, dtype)


def effective_sample_size(x, chunk=512, dtype=torch.float64):
    """diagnostics.py:158-203 on the device."""
    if x.shape[1] < 2:
        raise ValueError("effective_sample_size needs at least 2 draws")
    return _apply(x, _ess, chunk, dtype)


def rank_normalize(x, chunk=512, dtype=torch.float64):
    """z-scores of pooled average ranks of x [chains, draws, ...], per coordinate."""
    out = torch.cat([_rank_normalize(t) for t in _blocks(x, chunk, dtype)], dim=2)
    return out.reshape(x.shape)


def _bulk(t):
    z = _rank_normalize(_split(t))
    total = z.shape[0] * z.shape[1]
    tau = total / _ess(z)
    floor = 1.0 / math.log10(total)
    ok = torch.isfinite(tau) & (tau > 0)
    tau = torch.where(ok, torch.clamp(tau, min=floor), torch.full_like(tau, floor))
    return total / tau


def bulk_effective_sample_size(x, chunk=512, dtype=torch.float64):
    """Rank-normalised split-chain ESS on the device (``diagnostics.bulk_effective_sample_size``)."""
    return _apply(x, _bulk, chunk, dtype)


def mcse_mean(x, chunk=512, dtype=torch.float64):
    """sd / sqrt(ESS) per coordinate (``diagnostics.mcse_mean``)."""
    def f(t):
        flat = t.reshape(-1, t.shape[2])
        return flat.std(dim=0, unbiased=True) / torch.sqrt(_ess(t))
    return _apply(x, f, chunk, dtype)


def mcse_sd(x, chunk=512, dtype=torch.float64):
    """Delta-method MCSE of the sd from the ESS of the squared deviations (``diagnostics.mcse_sd``)."""
    def f(t):
        flat = t.reshape(-1, t.shape[2])
        m = flat.mean(dim=0)
        sd = flat.std(dim=0, unbiased=True)
        d2 = (t - m) ** 2
        var_d2 = d2.reshape(-1, t.shape[2]).var(dim=0, unbiased=True)
        return torch.sqrt(var_d2 / _ess(d2)) / (2.0 * sd)
    return _apply(x, f, chunk, dtype)


def summary_stats(x, chunk=512, dtype=torch.float64):
    """Per-coordinate mean, sd, bulk-ESS, numpyro ESS and split R-hat of x [chains, draws, ...]
    in one pass over the coordinates; a dict of tensors on x's device."""
    keys = ("mean", "std", "bulk_ess", "n_eff", "r_hat")
    parts = {k: [] for k in keys}
    for t in _blocks(x, chunk, dtype):
        flat = t.reshape(-1, t.shape[2])
        parts["mean"].append(flat.mean(dim=0))
        parts["std"].append(flat.std(dim=0, unbiased=True))
        parts["bulk_ess"].append(_bulk(t))
        parts["n_eff"].append(_ess(t))
        parts["r_hat"].append(_gelman_rubin(_split(t)))
    tail = tuple(x.shape[2:])
    return {k: torch.cat(v).reshape(tail) for k, v in parts.items()}


def hpdi(x, prob=0.90):
    """Highest posterior density interval of x [draws, ...] along its first dimension
    (numpyro/diagnostics.py:206-232), on x's device; [2, ...]."""
    sorted_x, _ = torch.sort(x, dim=0)
    mass = x.shape[0]
    index_length = int(prob * mass)
    lengths = sorted_x[index_length:] - sorted_x[: mass - index_length]
    start = torch.argmin(lengths, dim=0, keepdim=True)
    return torch.cat([torch.gather(sorted_x, 0, start), torch.gather(sorted_x, 0, start + index_length)], dim=0)


def summary(samples, prob=0.90, group_by_chain=True):
    """numpyro's summary (diagnostics.py:235-287) of torch tensors on the device: dict site ->
    {mean, std, median, hpdi bounds, n_eff, r_hat} as host numpy arrays (the per-coordinate
    results are all that leave the device)."""
    if not isinstance(samples, dict):
        samples = {"Param:{}".format(i): v for i, v in enumerate(samples)}
    out = {}
    for name, value in samples.items():
        if not group_by_chain:
            value = value.unsqueeze(0)
        flat = value.reshape((-1,) + tuple(value.shape[2:])).to(torch.float64)
        hpd = hpdi(flat, prob=prob)
        lo, hi = 50 * (1 - prob), 50 * (1 + prob)
        nan = torch.full_like(flat[0], float("nan"))
        st = {"mean": flat.mean(dim=0), "std": flat.std(dim=0, unbiased=True),
              "median": torch.sort(flat, dim=0).values[(flat.shape[0] - 1) // 2] if flat.shape[0] % 2 else
              torch.sort(flat, dim=0).values[flat.shape[0] // 2 - 1:flat.shape[0] // 2 + 1].mean(dim=0),
              "{:.1f}%".format(lo): hpd[0], "{:.1f}%".format(hi): hpd[1],
              "n_eff": effective_sample_size(value) if value.shape[1] >= 2 else nan,
              "r_hat": split_gelman_rubin(value) if value.shape[1] >= 4 else nan}
        out[name] = {k: v.detach().cpu().numpy() for k, v in st.items()}
    return out
