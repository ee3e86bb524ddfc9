"""gbn_sample_async: one transition for every chain enqueued without host synchronisation.

numpyro calls ``sample`` inside ``jit`` (numpyro/infer/mcmc.py:188-190, util.py:386-403), so
behind an XLA FFI call the transition must not block the host.  gbn_sample_async runs the tick
engine's loop on the device (a CUDA-graph WHILE node over batches of ticks, bounded by a tick
budget) and the hierarchical / stochastic-volatility families as one persistent launch.  It
must give exactly the states of the synchronous gbn_sample, through warmup (adaptation, window
ends) and sampling, for every engine path.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import NUTS, datasets, models  # noqa: E402

SEED = 97


def _case(name):
    if name == "hier":
        y, s = datasets.eight_schools(0)
        return models.HierarchicalNormal(y, s), 16, {}
    if name in ("logreg_fp32", "logreg_bf16x3"):
        X, y, _ = datasets.covtype_like(seed=2, n=20_000)
        return models.LogisticRegression(X, y), 128, {"precision": name.split("_")[1]}
    if name == "sv":
        r, _ = datasets.sv_returns(seed=1, T=512)
        return models.StochasticVolatility(r), 8, {}
    X, y, _ = datasets.horseshoe_data(seed=1, n=300, p=80, nonzero=4)
    return models.HorseshoeRegression(X, y, noncentered=True), 32, {"precision": "bf16x3"}


def _leaves(st):
    a = st.adapt_state
    return [st.i, st.z, st.z_grad, st.potential_energy, st.energy, st.num_steps, st.accept_prob,
            st.mean_accept_prob, st.diverging, a.step_size, a.inverse_mass_matrix, a.mass_matrix_sqrt,
            a.mass_matrix_sqrt_inv, a.ss_state, a.mm_state[0], a.mm_state[1], a.mm_state[2], a.window_idx,
            st.rng_key]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["hier", "logreg_fp32", "logreg_bf16x3", "sv", "horseshoe_bf16x3"])
def test_sample_async_is_bit_identical_to_sample(name):
    model, C, kw = _case(name)
    num_warmup, iters = 30, 40  # across the first window ends and into sampling
    k1 = NUTS(model, num_chains=C, **kw)
    k2 = NUTS(model, num_chains=C, **kw)
    s1 = k1.init(SEED, num_warmup)
    s2 = k2.init(SEED, num_warmup)
    for _ in range(iters):
        s1 = k1.sample(s1)
        s2 = k2.sample_async(s2)
    k2.check_async()
    torch.cuda.synchronize()
    for a, b in zip(_leaves(s1), _leaves(s2)):
        np.testing.assert_array_equal(a.cpu().numpy(), b.cpu().numpy())
    assert int(s2.i[0]) == iters
    k1.close()
    k2.close()
