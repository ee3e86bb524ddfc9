"""MCMC driver on the GPU: API contract (numpyro/infer/mcmc.py) and posterior
moments against the FP64 oracle (within 3 Monte-Carlo standard errors)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import MCMC, NUTS, HMC, datasets, diagnostics, models  # noqa: E402
from oracle import nuts_ref as R  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402


def _mcse_ok(gpu, ref, k=3.0):
    """|mean_gpu - mean_ref| within k * sqrt(mcse_gpu^2 + mcse_ref^2), per coordinate."""
    m1, m2 = gpu.mean(axis=(0, 1)), ref.mean(axis=(0, 1))
    s1, s2 = gpu.std(axis=(0, 1)), ref.std(axis=(0, 1))
    e1 = np.array([diagnostics.effective_sample_size(gpu[..., d]) for d in range(gpu.shape[-1])])
    e2 = np.array([diagnostics.effective_sample_size(ref[..., d]) for d in range(ref.shape[-1])])
    mcse = np.sqrt(s1 ** 2 / e1 + s2 ** 2 / e2)
    return np.abs(m1 - m2) <= k * mcse + 1e-6, m1, m2, mcse


@pytest.mark.gpu
def test_mcmc_api_eight_schools():
    y, s = datasets.eight_schools(0)
    model = models.HierarchicalNormal(y, s)
    mcmc = MCMC(NUTS(model), num_warmup=300, num_samples=400, num_chains=4)
    mcmc.run(0, extra_fields=("num_steps", "accept_prob", "adapt_state.step_size"))
    samples = mcmc.get_samples()
    assert samples["mu"].shape == (1600, 1) and samples["theta_base"].shape == (1600, 8)
    assert np.all(samples["tau"] > 0)
    grouped = mcmc.get_samples(group_by_chain=True)
    assert grouped["mu"].shape == (4, 400, 1)
    extra = mcmc.get_extra_fields()
    assert extra["num_steps"].shape == (1600,) and extra["diverging"].shape == (1600,)
    assert np.all(extra["num_steps"] >= 1)
    assert 0.5 < extra["accept_prob"].mean() <= 1.0
    assert np.all(np.diff(extra["adapt_state.step_size"].reshape(4, 400), axis=1) == 0)
    mcmc.print_summary()
    # warmup() then run() resumes from post_warmup_state without adapting
    m2 = MCMC(NUTS(model), num_warmup=200, num_samples=100, num_chains=4)
    m2.warmup(1)
    st = m2.post_warmup_state
    assert int(st.i[0]) == 200
    m2.run(2)
    assert m2.get_samples()["mu"].shape == (400, 1)
    assert int(m2.last_state.i[0]) == 300


@pytest.mark.gpu
def test_mcmc_keeps_draws_on_the_device_and_summarises_them_there(capsys):
    """keep_on_device=True: the same draws as the host-copy run, as CUDA tensors; print_summary's
    statistics (device_diagnostics) equal the host ones; transfer_states_to_host moves them."""
    from numpyro_gb300 import device_diagnostics as DD
    from numpyro_gb300 import diagnostics as D

    y, s = datasets.eight_schools(0)
    model = models.HierarchicalNormal(y, s)
    host = MCMC(NUTS(model), num_warmup=200, num_samples=300, num_chains=4)
    host.run(3)
    dev = MCMC(NUTS(model), num_warmup=200, num_samples=300, num_chains=4, keep_on_device=True)
    dev.run(3)
    hs, ds = host.get_samples(group_by_chain=True), dev.get_samples(group_by_chain=True)
    for k in hs:
        assert ds[k].is_cuda, k
        # the same unconstrained draws; exp of the positive sites by the device's own exp
        # (theta = mu + tau theta_base cancels: an ulp of tau's exp shows as ~1e-6 absolute)
        np.testing.assert_allclose(ds[k].cpu().numpy(), hs[k], rtol=1e-5, atol=1e-5, err_msg=k)
    assert dev.get_extra_fields()["diverging"].dtype == torch.bool
    a, b = D.summary({k: ds[k].cpu().double().numpy() for k in ds}), DD.summary(ds)  # both in FP64
    for site in a:
        for stat in a[site]:
            np.testing.assert_allclose(b[site][stat], np.asarray(a[site][stat]), rtol=1e-9, atol=1e-9,
                                       err_msg="%s %s" % (site, stat))
    dev.print_summary()
    assert "theta_base" in capsys.readouterr().out
    dev.transfer_states_to_host()
    assert isinstance(dev.get_samples()["mu"], np.ndarray)


@pytest.mark.gpu
def test_eight_schools_posterior_matches_oracle():
    y, s = datasets.eight_schools(0)
    model = models.HierarchicalNormal(y, s)
    C, W, S = 4, 500, 1000
    mcmc = MCMC(NUTS(model), num_warmup=W, num_samples=S, num_chains=C)
    mcmc.run(7)
    g = mcmc.get_samples(group_by_chain=True)
    zg = np.concatenate([g["mu"], np.log(g["tau"]), g["theta_base"]], axis=-1)  # unconstrained layout
    pot = PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))
    ref = np.array([R.run_chain(pot, model.latent_dim, 99, c, W, S)[0] for c in range(C)])
    ok, m1, m2, mcse = _mcse_ok(zg, ref)
    assert ok.mean() >= 0.9, (m1, m2, mcse)
    rhat = diagnostics.split_gelman_rubin(zg)
    assert np.all(rhat < 1.05), rhat


@pytest.mark.gpu
def test_logistic_posterior_plain_and_fused():
    X, yv, beta = datasets.covtype_like(seed=3, n=3000, n_cont=3, n_bin=3)
    model = models.LogisticRegression(X, yv)
    res = {}
    for engine in ["fused", "plain"]:
        mcmc = MCMC(NUTS(model, engine=engine), num_warmup=300, num_samples=500, num_chains=16)
        mcmc.run(3)
        res[engine] = mcmc.get_samples(group_by_chain=True)["coefs"]
    np.testing.assert_array_equal(res["fused"], res["plain"])
    pot = PR.make_potential("logreg", X.astype(np.float64), yv.astype(np.float64))
    ref = np.array([R.run_chain(pot, X.shape[1], 5, c, 300, 500)[0] for c in range(4)])
    ok, m1, m2, mcse = _mcse_ok(res["fused"], ref)
    assert ok.mean() >= 0.85, (m1, m2, mcse)
    assert np.all(diagnostics.split_gelman_rubin(res["fused"]) < 1.05)


@pytest.mark.gpu
def test_hmc_kernel_runs_and_adapts():
    y, s = datasets.eight_schools(0)
    model = models.HierarchicalNormal(y, s)
    mcmc = MCMC(HMC(model, trajectory_length=1.5), num_warmup=200, num_samples=200, num_chains=8)
    mcmc.run(4, extra_fields=("accept_prob",))
    acc = mcmc.get_extra_fields()["accept_prob"]
    assert 0.5 < acc.mean() <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["horseshoe", "horseshoe_nc", "sv"])
def test_large_latent_families_run(name):
    if name.startswith("horseshoe"):
        X, yh, beta = datasets.horseshoe_data(seed=1, n=300, p=60, nonzero=4)
        model = models.HorseshoeRegression(X, yh, noncentered=name.endswith("_nc"))
    else:
        r, _ = datasets.sv_returns(seed=1, T=600)
        model = models.StochasticVolatility(r)
    mcmc = MCMC(NUTS(model, max_tree_depth=8), num_warmup=150, num_samples=100, num_chains=8)
    mcmc.run(1, extra_fields=("accept_prob",))
    samp = mcmc.get_samples()
    for v in samp.values():
        assert np.all(np.isfinite(v))
    assert mcmc.get_extra_fields()["accept_prob"].mean() > 0.3


@pytest.mark.gpu
def test_logistic_bf16x3_engine_posterior():
    from numpyro_gb300 import _lib

    if not _lib.load().gbn_tc_available():
        pytest.skip("tcgen05 path needs an sm_103 GPU")
    X, yv, beta = datasets.covtype_like(seed=3, n=3000, n_cont=3, n_bin=3)
    model = models.LogisticRegression(X, yv)
    res = {}
    for prec in ["fp32", "bf16x3"]:
        mcmc = MCMC(NUTS(model, precision=prec), num_warmup=300, num_samples=500, num_chains=128)
        mcmc.run(3)
        res[prec] = mcmc.get_samples(group_by_chain=True)["coefs"]
    ok, m1, m2, mcse = _mcse_ok(res["bf16x3"], res["fp32"])
    assert ok.mean() >= 0.85, (m1, m2, mcse)
    assert np.all(diagnostics.split_gelman_rubin(res["bf16x3"]) < 1.02)


@pytest.mark.gpu
def test_functional_hmc_api_matches_the_kernel_class():
    """hmc(potential, algo="NUTS") + fori_collect (numpyro/infer/hmc.py:113, numpyro/util.py:321),
    as examples/stochastic_volatility.py drives it, gives the NUTS class's draws bit for bit."""
    from numpyro_gb300 import NUTS, datasets, fori_collect, hmc, models

    ys, ss = datasets.eight_schools(0)
    model = models.HierarchicalNormal(ys, ss)
    init_kernel, sample_kernel = hmc(model, algo="NUTS", num_chains=4)
    st = init_kernel(None, 0, step_size=0.3, adapt_step_size=False, adapt_mass_matrix=False, rng_key=2024)
    draws = fori_collect(1, 4, sample_kernel, st, transform=lambda s: s.z)
    k = NUTS(model, num_chains=4, step_size=0.3, adapt_step_size=False, adapt_mass_matrix=False)
    s = k.init(2024, 0)
    ref = []
    for _ in range(4):
        s = k.sample(s)
        ref.append(s.z.cpu().numpy())
    assert draws.shape == (3, 4, model.latent_dim)
    np.testing.assert_array_equal(draws, np.stack(ref[1:]))
    k.close()
    init_kernel.kernel().close()
