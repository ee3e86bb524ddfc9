"""Diagnostics contracts of numpyro's test/test_diagnostics.py:19-59 (shapes, batching along the
last axis, HPDI), on seeded inputs, and the keys of summary() (numpyro/diagnostics.py:235-287)."""
import numpy as np
import pytest

from numpyro_gb300.diagnostics import (autocorrelation, autocovariance, effective_sample_size, gelman_rubin, hpdi,
                                       split_gelman_rubin, summary)


@pytest.mark.parametrize("statistic, input_shape, output_shape", [
    (autocorrelation, (10,), (10,)), (autocorrelation, (10, 3), (10, 3)),
    (autocovariance, (10,), (10,)), (autocovariance, (10, 3), (10, 3)),
    (hpdi, (10,), (2,)), (hpdi, (10, 3), (2, 3)),
    (gelman_rubin, (4, 10), ()), (gelman_rubin, (4, 10, 3), (3,)),
    (split_gelman_rubin, (4, 10), ()), (split_gelman_rubin, (4, 10, 3), (3,)),
    (effective_sample_size, (4, 10), ()), (effective_sample_size, (4, 10, 3), (3,)),
])
def test_shape_and_batching(statistic, input_shape, output_shape):
    x = np.random.default_rng(0).normal(size=input_shape)
    y = statistic(x)
    assert np.shape(y) == output_shape
    if x.shape[-1] == 3:  # the last axis is a batch: each column alone gives the same values
        for i in range(3):
            np.testing.assert_allclose(statistic(x[..., i]), y[..., i])


def test_hpdi():
    """numpyro's test_hpdi (test_diagnostics.py:53-58).  For the normal its 20,000 draws and 0.01
    tolerance are within the statistic's own noise (the narrowest 80 % window of a normal sample
    wanders by up to ~0.1 from the central quantiles at that size, shrinking about as n^-1/3), so
    the normal case uses 10^6 draws and 0.03.  The exponential case, anchored at 0, keeps 0.01."""
    rng = np.random.default_rng(1)
    x = rng.normal(size=1_000_000)
    np.testing.assert_allclose(hpdi(x, prob=0.8), np.quantile(x, [0.1, 0.9]), atol=0.03)
    x = rng.exponential(size=20000)
    np.testing.assert_allclose(hpdi(x, prob=0.2), [0.0, 0.22], atol=0.01)


def test_hpdi_is_the_narrowest_window():
    """Brute force over every window of int(prob * n) + 1 sorted draws (diagnostics.py:206-232)."""
    rng = np.random.default_rng(3)
    for x in (rng.gamma(2.0, size=301), rng.standard_t(3, size=200)):
        s = np.sort(x)
        k = int(0.7 * x.size)
        lengths = [s[i + k] - s[i] for i in range(x.size - k)]
        i = int(np.argmin(lengths))
        np.testing.assert_array_equal(hpdi(x, prob=0.7), [s[i], s[i + k]])


def test_summary_keys_and_values():
    rng = np.random.default_rng(2)
    s = summary({"a": rng.normal(size=(4, 500)), "b": rng.normal(size=(4, 500, 2))}, prob=0.9)
    assert list(s["a"]) == ["mean", "std", "median", "5.0%", "95.0%", "n_eff", "r_hat"]
    assert s["b"]["mean"].shape == (2,)
    assert abs(float(s["a"]["mean"])) < 0.1 and abs(float(s["a"]["std"]) - 1) < 0.1
    assert 0.99 < float(s["a"]["r_hat"]) < 1.01
    flat = summary({"a": rng.normal(size=(2000,))}, group_by_chain=False)
    assert flat["a"]["n_eff"] > 1000


def test_mcse_of_mean_and_sd_on_independent_normal_draws():
    """Known answers: for independent N(0, 1) draws the standard errors of the mean and of the sd
    are 1 / sqrt(N) and 1 / sqrt(2 N)."""
    from numpyro_gb300.diagnostics import mcse_mean, mcse_sd

    x = np.random.default_rng(0).standard_normal((8, 2000, 4))
    n = 8 * 2000
    np.testing.assert_allclose(mcse_mean(x), 1 / np.sqrt(n), rtol=0.1)
    np.testing.assert_allclose(mcse_sd(x), 1 / np.sqrt(2 * n), rtol=0.1)


def test_posterior_gate_bounds():
    """The chance allowance of the posterior gates (tests/test_gpu_posterior_gates.py): independent
    standard-normal z-scores pass it about 99 % of the time."""
    import importlib.util
    import os

    pytest.importorskip("torch")
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "test_gpu_posterior_gates.py")
    spec = importlib.util.spec_from_file_location("gates_under_test", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    b3, bound = mod.moment_bounds(110)
    assert b3 == 2 and abs(bound - 3.91) < 0.01
    b3, bound = mod.moment_bounds(1028)
    assert b3 == 8 and abs(bound - 4.42) < 0.01
    z = np.abs(np.random.default_rng(1).standard_normal((2000, 110)))
    b3, bound = mod.moment_bounds(110)
    ok = (np.sum(z > 3, axis=1) <= b3) & (z.max(axis=1) <= bound)
    assert ok.mean() > 0.97


def _ar1_draws_with_ties(C, S, K, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros((C, S, K))
    e = rng.standard_normal((C, S, K))
    for s in range(S):
        x[:, s] = 0.6 * x[:, s - 1] + e[:, s] if s else e[:, s]
    stay = rng.random((C, S)) < 0.2  # rejected transitions repeat their draw
    for c in range(C):
        for s in range(1, S):
            if stay[c, s]:
                x[c, s] = x[c, s - 1]
    x[:, :, 3] = np.round(x[:, :, 3])  # a coordinate of heavy ties
    return x


def test_device_diagnostics_equal_the_host_estimators():
    """device_diagnostics (torch, here on CPU tensors: the same code runs on the GPU) against the
    host restatement of numpyro's estimators, with ties and in chunks that split the coordinates."""
    torch = pytest.importorskip("torch")
    from numpyro_gb300 import device_diagnostics as DD
    from numpyro_gb300 import diagnostics as D

    x = _ar1_draws_with_ties(8, 301, 37)
    t = torch.as_tensor(x)
    for name in ("split_gelman_rubin", "gelman_rubin", "effective_sample_size", "bulk_effective_sample_size",
                 "mcse_mean", "mcse_sd"):
        a, b = getattr(D, name)(x), getattr(DD, name)(t, chunk=10).numpy()
        np.testing.assert_allclose(b, a, rtol=1e-12, err_msg=name)
    np.testing.assert_allclose(DD.rank_normalize(t, chunk=7).numpy(), D.rank_normalize(x), atol=1e-12)
    hs, ds = D.summary({"a": x}), DD.summary({"a": t})
    for k in hs["a"]:
        np.testing.assert_allclose(ds["a"][k], np.asarray(hs["a"][k]), rtol=1e-12, atol=1e-14, err_msg=k)
    st = DD.summary_stats(t, chunk=9)
    np.testing.assert_allclose(st["bulk_ess"].numpy(), D.bulk_effective_sample_size(x), rtol=1e-12)
    np.testing.assert_allclose(st["r_hat"].numpy(), D.split_gelman_rubin(x), rtol=1e-12)


def test_device_diagnostics_on_a_model_major_view():
    """Per-model statistics of a batch of models without copying the draws: the chains of model m
    are rows 4m..4m+3, viewed as [4 chains, draws, models, coordinates]."""
    torch = pytest.importorskip("torch")
    from numpyro_gb300 import device_diagnostics as DD
    from numpyro_gb300 import diagnostics as D

    y = _ar1_draws_with_ties(6 * 4, 120, 5, seed=3)
    yt = torch.as_tensor(y).view(6, 4, 120, 5).permute(1, 2, 0, 3)
    ref = np.stack([D.bulk_effective_sample_size(y[4 * m:4 * m + 4]) for m in range(6)])
    np.testing.assert_allclose(DD.bulk_effective_sample_size(yt, chunk=7).numpy(), ref, rtol=1e-12)
    ref = np.stack([D.split_gelman_rubin(y[4 * m:4 * m + 4]) for m in range(6)])
    np.testing.assert_allclose(DD.split_gelman_rubin(yt, chunk=3).numpy(), ref, rtol=1e-12)
