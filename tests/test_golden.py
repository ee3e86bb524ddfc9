"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the FP64 oracle)."""
import os

import numpy as np
import pytest

from oracle import nuts_ref as R
from oracle import potentials_ref as PR

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_oracle_reproduces_golden_warmup_trajectories():
    g = _load("nuts_hier_nc_warmup.npz")
    pot = PR.make_potential("hier_nc", g["y"].astype(np.float64), g["sigma"].astype(np.float64))
    seed = int(g["seed"])
    for c in range(g["z0"].shape[0]):
        init_kernel, sample_kernel = R.hmc(pot)
        st = init_kernel(g["z0"][c], 50, rng_key=(seed, c))
        for t in range(g["z"].shape[1]):
            st = sample_kernel(st)
            assert st.num_steps == g["num_steps"][c, t]
            np.testing.assert_allclose(st.z, g["z"][c, t], rtol=1e-12, atol=1e-12)


def test_oracle_reproduces_golden_potentials():
    g = _load("potential_logreg.npz")
    X, y = g["X"].astype(np.float64), g["y"].astype(np.float64)
    for k in range(g["z"].shape[0]):
        np.testing.assert_allclose(PR.logreg_potential(g["z"][k], X, y), g["pe"][k], rtol=1e-13)
        np.testing.assert_allclose(PR.logreg_grad(g["z"][k], X, y), g["grad"][k], rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_gpu_first_warmup_transitions_match_golden():
    """The CUDA engine reproduces the golden tree sizes of the first warmup transitions
    (identical Philox bits; later transitions may part by FP32-vs-FP64 chaos)."""
    torch = pytest.importorskip("torch")
    from numpyro_gb300 import NUTS, models

    g = _load("nuts_hier_nc_warmup.npz")
    C = g["z0"].shape[0]
    k = NUTS(models.HierarchicalNormal(g["y"], g["sigma"]), num_chains=C)
    st = k.init(int(g["seed"]), 50)
    np.testing.assert_allclose(st.z.cpu().numpy(), g["z0"], rtol=1e-6, atol=1e-6)
    for t in range(3):
        st = k.sample(st)
        np.testing.assert_array_equal(st.num_steps.cpu().numpy(), g["num_steps"][:, t])
        np.testing.assert_allclose(st.z.cpu().numpy(), g["z"][:, t], rtol=1e-4, atol=1e-4)
    k.close()


@pytest.mark.gpu
def test_gpu_logreg_potential_matches_golden():
    torch = pytest.importorskip("torch")
    from numpyro_gb300 import NUTS, models
    from numpyro_gb300.torch_ops import potential

    g = _load("potential_logreg.npz")
    k = NUTS(models.LogisticRegression(g["X"], g["y"]), num_chains=g["z"].shape[0])
    z = torch.tensor(g["z"], dtype=torch.float32, device="cuda", requires_grad=True)
    pe = potential(k, z)
    pe.sum().backward()
    np.testing.assert_allclose(pe.detach().cpu().numpy(), g["pe"], rtol=2e-6)
    np.testing.assert_allclose(z.grad.cpu().numpy(), g["grad"], atol=1e-3 * np.abs(g["grad"]).max())
    k.close()
