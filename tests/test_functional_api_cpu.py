"""The functional API on the host: fori_collect (numpyro/util.py:321-454) and hmc()
(numpyro/infer/hmc.py:113-538).  The device calls of the kernels are replaced by stubs here; the
kernels themselves are covered by the GPU tests."""
from collections import namedtuple

import numpy as np
import pytest


def test_fori_collect_slots_follow_the_reference():
    """util.py:370-395: start = lower + (upper - lower) % thinning, and iteration i writes slot
    (i - start) // thinning when >= 0, so each slot keeps the last value of its thinning group."""
    from numpyro_gb300 import fori_collect

    out = fori_collect(2, 10, lambda x: x + 1, np.zeros(3), thinning=3)
    # start = 2 + 8 % 3 = 4; slot 0 <- i = 4, 5, 6 (value after i = 6 is 7); slot 1 <- i = 7, 8, 9 (10)
    np.testing.assert_array_equal(out[:, 0], [7.0, 10.0])
    out = fori_collect(3, 7, lambda x: x + 1, np.zeros(2))
    np.testing.assert_array_equal(out[:, 0], [4.0, 5.0, 6.0, 7.0])


@pytest.mark.parametrize("lower,upper,thinning,expected", [
    (0, 9, 2, [2, 4, 6, 8]), (0, 9, 3, [2, 5, 8]), (0, 9, 4, [4, 8]), (12, 37, 5, [16, 21, 26, 31, 36])])
def test_fori_collect_thinning_known_answers(lower, upper, thinning, expected):
    """The known answers of numpyro's test/test_util.py:18-36 (x -> x + 1 from [-1])."""
    from numpyro_gb300 import fori_collect

    out = fori_collect(lower, upper, lambda x: x + 1, np.array([-1]), thinning=thinning)
    np.testing.assert_array_equal(out[:, 0], expected)


def test_fori_collect_tree_and_last_value_known_answers():
    """numpyro's test/test_util.py:39-68: a dict carry with a transform, and return_last_val."""
    from numpyro_gb300 import fori_collect

    def f(x):
        return {"i": x["i"] + x["j"], "j": x["i"] - x["j"]}

    out = fori_collect(1, 3, f, {"i": np.array([0.0]), "j": np.array([1.0])}, transform=lambda a: {"i": a["i"]})
    np.testing.assert_array_equal(out["i"], [[0.0], [2.0]])

    def g(x):
        x["i"] = x["i"] + 1
        return x

    tree, last = fori_collect(2, 4, g, {"i": 0}, transform=lambda a: {"i": a["i"]}, return_last_val=True)
    np.testing.assert_array_equal(tree["i"], [3, 4])
    assert last["i"] == 4


def test_fori_collect_structures_transform_and_last_value():
    from numpyro_gb300 import fori_collect

    S = namedtuple("S", ["a", "b", "c"])
    init = S(np.zeros(2), {"u": np.ones(())}, None)

    def body(s):
        return S(s.a + 1, {"u": s.b["u"] * 2}, None)

    coll, last = fori_collect(0, 4, body, init, return_last_val=True, collection_size=6)
    assert isinstance(coll, S) and coll.c is None
    assert coll.a.shape == (6, 2) and coll.b["u"].shape == (6,)
    np.testing.assert_array_equal(coll.a[:, 0], [1, 2, 3, 4, 0, 0])
    np.testing.assert_array_equal(coll.b["u"], [2, 4, 8, 16, 0, 0])
    np.testing.assert_array_equal(last.a, [4, 4])
    only_a = fori_collect(1, 4, body, init, transform=lambda s: s.a)
    assert only_a.shape == (3, 2)


def test_hmc_functional_api_builds_and_steps_the_kernel(monkeypatch):
    from numpyro_gb300 import HMC, NUTS, hmc, models

    calls = []

    def fake_init(self, rng_key, num_warmup, init_params=None, model_args=(), model_kwargs={}):
        calls.append(("init", type(self).__name__, rng_key, num_warmup,
                      None if init_params is None else np.asarray(init_params).shape))
        return "state0"

    def fake_sample(self, state, model_args=(), model_kwargs={}):
        calls.append(("sample", state))
        return state + "'"

    monkeypatch.setattr(HMC, "init", fake_init)
    monkeypatch.setattr(HMC, "sample", fake_sample)
    model = models.HierarchicalNormal(np.zeros(3), np.ones(3))
    init_kernel, sample_kernel = hmc(model, algo="NUTS", num_chains=4)
    st = init_kernel(np.zeros(model.latent_dim), 50, step_size=0.3, max_tree_depth=7, rng_key=11)
    k = init_kernel.kernel()
    assert isinstance(k, NUTS) and k._max_tree_depth == 7 and k._step_size == pytest.approx(0.3)
    assert calls[0] == ("init", "NUTS", 11, 50, (4, model.latent_dim))  # one start broadcast to 4 chains
    assert sample_kernel(st) == "state0'"
    init_kernel, sample_kernel = hmc(model, algo="HMC")
    init_kernel(None, 10, num_steps=5, trajectory_length=None, rng_key=np.zeros((3, 2), np.uint32))
    k = init_kernel.kernel()
    assert type(k) is HMC and k._num_steps == 5
    assert calls[-1][:2] == ("init", "HMC") and calls[-1][4] is None


def test_hmc_functional_api_rejects_what_the_engine_cannot_run():
    from numpyro_gb300 import hmc, models

    model = models.HierarchicalNormal(np.zeros(3), np.ones(3))
    with pytest.raises(ValueError):
        hmc(model, algo="SA")
    with pytest.raises(NotImplementedError):
        hmc(lambda z: z)
    with pytest.raises(NotImplementedError):
        hmc(model, kinetic_fn=lambda inv, r: 0.0)
    _, sample_kernel = hmc(model)
    with pytest.raises(RuntimeError):
        sample_kernel(None)


def test_initialize_model_feeds_the_functional_api(monkeypatch):
    """The flow of examples/stochastic_volatility.py:90-107 with a registry model: initialize_model
    -> hmc(model_info.potential_fn) -> init_kernel(model_info.param_info) -> fori_collect with
    postprocess_fn (the device calls stubbed)."""
    import torch

    from numpyro_gb300 import HMC, fori_collect, hmc, initialize_model, models

    T = 6
    model = models.StochasticVolatility(np.linspace(-0.01, 0.01, T))
    info = initialize_model(0, model, model_args=())
    assert info.potential_fn is model and info.param_info.z is None and info.model_trace is None

    class _S:
        def __init__(self, z):
            self.z = z

    seen = {}

    def fake_init(self, rng_key, num_warmup, init_params=None, model_args=(), model_kwargs={}):
        seen["init_params"] = init_params
        return _S(torch.zeros(1, model.latent_dim))

    monkeypatch.setattr(HMC, "init", fake_init)
    monkeypatch.setattr(HMC, "sample", lambda self, s, model_args=(), model_kwargs={}: _S(s.z + 0.1))
    init_kernel, sample_kernel = hmc(info.potential_fn, algo="NUTS")
    state = init_kernel(info.param_info, 3, rng_key=1)
    assert seen["init_params"] is None  # no starting point: drawn on the device
    out = fori_collect(3, 5, sample_kernel, state, transform=lambda s: info.postprocess_fn(s.z.numpy()))
    assert sorted(out) == ["h", "nu", "s"] and out["h"].shape == (2, 1, T)
    np.testing.assert_allclose(out["s"][:, 0, 0], np.exp([0.4, 0.5]), rtol=1e-6)
    with pytest.raises(NotImplementedError):
        initialize_model(0, lambda: None)
