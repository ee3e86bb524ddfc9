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


def _terms(kernel):
    import ctypes

    from numpyro_gb300 import _lib

    three, blocks, limit = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_float()
    _lib.check(_lib.load().gbn_logreg_terms(kernel._handle, ctypes.byref(three), ctypes.byref(blocks),
                                            ctypes.byref(limit)), kernel._handle)
    return three.value, blocks.value, limit.value


def _lo2(z):
    """Sum over coefficients of the squared third bf16 term of z / 2 (the split's arithmetic)."""
    from numpyro_gb300.datasets import _round_bf16

    h = (0.5 * np.asarray(z, np.float32)).astype(np.float32)
    r1 = (h - _round_bf16(h)).astype(np.float32)
    r2 = (r1 - _round_bf16(r1)).astype(np.float32)
    return np.sum(r2.astype(np.float64) ** 2, axis=-1)


@pytest.mark.gpu
def test_logreg_tc_two_coefficient_terms_agree_with_three(monkeypatch):
    """The tensor-core kernel leaves out the third bf16 term of the coefficients when the
    first-order energy term added in its place is exact to 1e-3 (covtype-like data: the
    remainder bound is ~1e-7); its energies must then match the kernel run with all three
    terms (GBN_LOGREG_TERMS=3) and the FP64 oracle, and its limit must be 2e-3 over the
    Gershgorin bound on lambda_max(X^T X)."""
    _tc_or_skip()
    from numpyro_gb300 import datasets, models

    X, y, beta = datasets.covtype_like(seed=2, n=40_000)
    rng = np.random.default_rng(3)
    z = (beta[None, :] + 0.02 * rng.standard_normal((256, X.shape[1]))).astype(np.float32)
    zt = torch.as_tensor(z, device="cuda")
    k2 = NUTS(models.LogisticRegression(X, y), num_chains=256, precision="bf16x3")
    pe2, g2 = [t.cpu().numpy() for t in k2.potential_and_grad(zt)]
    three, blocks, limit = _terms(k2)
    k2.close()
    gram = X.T.astype(np.float64) @ X.astype(np.float64)
    lam = np.max(np.sum(np.abs(gram), axis=1))
    np.testing.assert_allclose(limit, 2e-3 / (1.01 * lam), rtol=1e-4)
    assert (three, blocks) == (0, 2), (three, blocks, limit, _lo2(z).max())
    monkeypatch.setenv("GBN_LOGREG_TERMS", "3")
    k3 = NUTS(models.LogisticRegression(X, y), num_chains=256, precision="bf16x3")
    pe3, g3 = [t.cpu().numpy() for t in k3.potential_and_grad(zt)]
    assert _terms(k3)[:2] == (2, 2)
    k3.close()
    print("two vs three terms: max |dU| %.3e (U ~ %.3e)" % (np.max(np.abs(pe2 - pe3)), np.abs(pe3).max()))
    assert np.max(np.abs(pe2 - pe3)) <= 2e-7 * np.abs(pe3).max() + 1e-3
    scale = np.max(np.abs(g3), axis=1, keepdims=True)
    assert np.max(np.abs(g2 - g3) / scale) < 3e-3
    X64, y64 = X.astype(np.float64), y.astype(np.float64)
    for c in (0, 101, 255):
        pr = PR.logreg_potential(z[c].astype(np.float64), X64, y64)
        assert abs(pe2[c] - pr) <= 1e-6 * abs(pr) + 1e-3, (c, pe2[c], pr)


@pytest.mark.gpu
def test_logreg_tc_takes_three_terms_where_a_block_needs_them(monkeypatch):
    """Coefficients of +-1000 on two identical columns in the chains of one 128-chain block only:
    their third bf16 terms (~4e-3) put that block over the limit, so it (and only it) takes all
    three terms, and gives what a run that always takes three gives (the gradient bit for bit; the
    energy to FP64 rounding, as a chain's four per-thread sums meet in FP64 shared-memory atomics)."""
    _tc_or_skip()
    from numpyro_gb300 import datasets, models

    rng = np.random.default_rng(11)
    n, p, C = 5000, 6, 256
    X = np.empty((n, p), np.float32)
    x = datasets._round_bf16(rng.standard_normal(n).astype(np.float32))
    X[:, 0] = x
    X[:, 1] = x
    X[:, 2:-1] = datasets._round_bf16(rng.standard_normal((n, p - 3)).astype(np.float32))
    X[:, -1] = 1.0
    y = (rng.random(n) < 0.5).astype(np.float32)
    z = (0.3 * rng.standard_normal((C, p))).astype(np.float32)
    big = (1000.0 + 3.0 * rng.random(128)).astype(np.float32)
    z[128:, 0] += big
    z[128:, 1] -= big
    zt = torch.as_tensor(z, device="cuda")
    model = models.LogisticRegression(X, y, prior_scale=2000.0)
    k = NUTS(model, num_chains=C, precision="bf16x3")
    pe, g = [t.cpu().numpy() for t in k.potential_and_grad(zt)]
    three, blocks, limit = _terms(k)
    k.close()
    lo2 = _lo2(z)
    print("limit %.3e; largest |lo|^2 block 0 %.3e, block 1 %.3e" % (limit, lo2[:128].max(), lo2[128:].max()))
    assert lo2[:128].max() <= limit < lo2[128:].max()
    assert (three, blocks) == (1, 2)
    monkeypatch.setenv("GBN_LOGREG_TERMS", "3")
    k3 = NUTS(model, num_chains=C, precision="bf16x3")
    pe3, g3 = [t.cpu().numpy() for t in k3.potential_and_grad(zt)]
    k3.close()
    np.testing.assert_allclose(pe[128:], pe3[128:], rtol=1e-13)
    np.testing.assert_array_equal(g[128:], g3[128:])


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
