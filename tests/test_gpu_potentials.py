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


# ---------------------------------------------------------------- tensor-core (tcgen05) logistic potential
def _tc_or_skip():
    from numpyro_gb300 import _lib

    if not _lib.load().gbn_tc_available():
        pytest.skip("tcgen05 path needs an sm_103 GPU")


@pytest.mark.gpu
@pytest.mark.parametrize("n,p,C", [(1000, 13, 200), (3000, 55, 128), (257, 64, 1), (5000, 7, 1030)])
def test_logreg_tc_matches_oracle(n, p, C):
    """bf16x3 tensor-core potential: U within 1e-6 relative of FP64, grad within 3e-3 of its scale."""
    _tc_or_skip()
    from numpyro_gb300 import datasets, models

    rng = np.random.default_rng(n + p)
    X = np.empty((n, p), np.float32)
    X[:, :-1] = datasets._round_bf16(rng.standard_normal((n, p - 1)).astype(np.float32)) if p > 1 else 0
    X[:, -1] = 1.0
    y = (rng.random(n) < 0.4).astype(np.float32)
    z = (0.3 * rng.standard_normal((C, p))).astype(np.float32)
    k = NUTS(models.LogisticRegression(X, y), num_chains=C, precision="bf16x3")
    pe, g = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    pe, g = pe.cpu().numpy(), g.cpu().numpy()
    X64, y64 = X.astype(np.float64), y.astype(np.float64)
    for c in sorted(set([0, C // 2, C - 1])):
        pr = PR.logreg_potential(z[c], X64, y64)
        gr = PR.logreg_grad(z[c], X64, y64)
        assert abs(pe[c] - pr) <= 1e-6 * abs(pr) + 1e-3, (c, pe[c], pr)
        np.testing.assert_allclose(g[c], gr, atol=3e-3 * np.max(np.abs(gr)) + 1e-3)
    k.close()


@pytest.mark.gpu
def test_logreg_tc_matches_fp32_path_full_size():
    """covtype-shaped N=581,012 x 55 with 1024 points: tensor-core vs FP32 CUDA-core potential."""
    _tc_or_skip()
    from numpyro_gb300 import datasets, models

    X, y, beta = datasets.covtype_like(seed=0)
    m = models.LogisticRegression(X, y)
    rng = np.random.default_rng(1)
    z = (beta[None, :] + 0.01 * rng.standard_normal((1024, X.shape[1]))).astype(np.float32)
    zt = torch.as_tensor(z, device="cuda")
    ktc = NUTS(m, num_chains=1024, precision="bf16x3")
    k32 = NUTS(m, num_chains=1024, precision="fp32")
    pe_tc, g_tc = [t.cpu().numpy() for t in ktc.potential_and_grad(zt)]
    pe_32, g_32 = [t.cpu().numpy() for t in k32.potential_and_grad(zt)]
    assert np.max(np.abs(pe_tc - pe_32) / np.abs(pe_32)) < 2e-7
    scale = np.max(np.abs(g_32), axis=1, keepdims=True)
    assert np.max(np.abs(g_tc - g_32) / scale) < 5e-3
    pr = PR.logreg_potential(z[5], X.astype(np.float64), y.astype(np.float64))
    assert abs(pe_tc[5] - pr) <= 2e-8 * abs(pr) + 0.05
    ktc.close()
    k32.close()


TUNED = [c for c in CASES if c[0] in ("hier_nc", "logreg", "horseshoe", "horseshoe_nc")]


@pytest.mark.gpu
@pytest.mark.parametrize("case", TUNED, ids=[c[0] for c in TUNED])
def test_autotuner_reports_its_choice(case):
    name, model, _ = case
    k = NUTS(model, num_chains=16)
    k.potential_and_grad(torch.as_tensor(typical_points(name, model, np.random.default_rng(0), 16), device="cuda"))
    assert "=" in k.tuning(), k.tuning()
    k.close()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", ["hs_tm=2 hs_splits=1", "hs_tm=2 hs_splits=8", "hs_tm=4 hs_splits=3"])
@pytest.mark.parametrize("name", ["horseshoe", "horseshoe_nc"])
def test_horseshoe_tile_shapes_agree_with_oracle(shape, name, monkeypatch):
    """Every tile height / split count the autotuner may pick gives the oracle's potential."""
    monkeypatch.setenv("GBN_TUNE", shape)
    _, model, ref = [c for c in CASES if c[0] == name][0]
    rng = np.random.default_rng(2)
    C = 21
    z = typical_points(name, model, rng, C)
    k = NUTS(model, num_chains=C)
    pe, g = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    assert k.tuning() == "horseshoe_tile_rows=%d horseshoe_splits=%d" % (16 * int(shape[6]), int(shape.split("=")[-1]))
    pe, g = pe.cpu().numpy(), g.cpu().numpy()
    for c in range(C):
        pr, gr = ref(z[c].astype(np.float64))
        assert abs(pe[c] - pr) <= 2e-6 * max(1.0, abs(pr)), (shape, c, pe[c], pr)
        np.testing.assert_allclose(g[c], gr, atol=1e-3 * max(1.0, np.max(np.abs(gr))), rtol=1e-3)
    k.close()


@pytest.mark.gpu
@pytest.mark.parametrize("noncentered", [False, True])
@pytest.mark.parametrize("shape", [(200, 50, 37), (333, 130, 130)])
def test_horseshoe_tensor_core_vs_oracle(shape, noncentered):
    """precision="bf16x3": both horseshoe GEMMs on tcgen05 (six bf16 cross products per split
    operand pair) match the FP64 oracle like the FP32 CUDA-core path."""
    _tc_or_skip()
    from numpyro_gb300 import datasets, models

    n, p, C = shape
    X, yh, _ = datasets.horseshoe_data(seed=9, n=n, p=p, nonzero=5)
    model = models.HorseshoeRegression(X, yh, noncentered=noncentered)
    name = "horseshoe_nc" if noncentered else "horseshoe"
    ref = PR.make_potential(name, X.astype(np.float64), yh.astype(np.float64))
    z = typical_points(name, model, np.random.default_rng(4), C)
    k = NUTS(model, num_chains=C, precision="bf16x3")
    pe, g = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    pe, g = pe.cpu().numpy(), g.cpu().numpy()
    for c in range(C):
        pr, gr = ref(z[c].astype(np.float64))
        assert abs(pe[c] - pr) <= 2e-6 * max(1.0, abs(pr)), (c, pe[c], pr)
        np.testing.assert_allclose(g[c], gr, atol=1e-3 * max(1.0, np.max(np.abs(gr))), rtol=1e-3)
    k.close()
