"""GPU potentials + hand-written adjoints vs the FP64 oracle (and central FD).

Tolerances: potential within 2e-6 relative of the FP64 closed form (FP32
terms, FP64 sums); gradients within 1e-3 of the gradient scale (FP32 GEMMs).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import NUTS  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402
from tests.gpu_helpers import family_cases, typical_points  # noqa: E402

CASES = family_cases()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_potential_and_grad_vs_oracle(case):
    name, model, ref = case
    rng = np.random.default_rng(11)
    C = 37
    z = typical_points(name, model, rng, C)
    k = NUTS(model, num_chains=C)
    pe, g = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    pe, g = pe.cpu().numpy(), g.cpu().numpy()
    for c in range(C):
        pr, gr = ref(z[c].astype(np.float64))
        assert abs(pe[c] - pr) <= 2e-6 * max(1.0, abs(pr)), (name, c, pe[c], pr)
        scale = max(1.0, np.max(np.abs(gr)))
        np.testing.assert_allclose(g[c], gr, atol=1e-3 * scale, rtol=1e-3, err_msg=name)
    k.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_adjoint_vs_central_fd(case):
    name, model, ref = case
    rng = np.random.default_rng(5)
    z = typical_points(name, model, rng, 1)[0].astype(np.float64)
    k = NUTS(model, num_chains=1)
    _, g = k.potential_and_grad(torch.as_tensor(z[None].astype(np.float32), device="cuda"))
    g = g.cpu().numpy()[0]
    f = lambda v: ref(v)[0]  # noqa: E731
    idx = rng.choice(z.size, min(z.size, 12), replace=False)
    for i in idx:
        e = np.zeros_like(z)
        e[i] = 1e-3
        fd = (f(z + e) - f(z - e)) / 2e-3
        assert abs(g[i] - fd) <= 2e-3 * max(1.0, abs(fd)), (name, i, g[i], fd)
    k.close()


@pytest.mark.gpu
def test_logreg_full_size_subset_of_chains():
    """covtype-shaped N=581,012 x 55: FP32 SIMT potential vs FP64 on 4 points."""
    from numpyro_gb300 import datasets, models

    X, y, beta = datasets.covtype_like(seed=0)
    m = models.LogisticRegression(X, y)
    rng = np.random.default_rng(0)
    z = (beta[None, :] + 0.01 * rng.standard_normal((4, X.shape[1]))).astype(np.float32)
    k = NUTS(m, num_chains=4)
    pe, g = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    pe, g = pe.cpu().numpy(), g.cpu().numpy()
    X64, y64 = X.astype(np.float64), y.astype(np.float64)
    for c in range(4):
        pr = PR.logreg_potential(z[c], X64, y64)
        gr = PR.logreg_grad(z[c], X64, y64)
        assert abs(pe[c] - pr) <= 1e-7 * abs(pr) + 1e-3, (pe[c], pr)
        np.testing.assert_allclose(g[c], gr, atol=2e-3 * np.max(np.abs(gr)) + 0.05)
    k.close()
