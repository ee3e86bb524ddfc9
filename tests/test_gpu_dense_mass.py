"""dense_mass=True: the device factorisation, dense transitions and dense Welford adaptation
against the FP64 oracle's restatement of numpyro (hmc_util.py:133-239, :439-515; hmc.py:92-110)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import MCMC, NUTS, datasets, diagnostics, models  # noqa: E402
from oracle import nuts_ref as R  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402

SEED = 4321


def _hier():
    y, s = datasets.eight_schools(0)
    return models.HierarchicalNormal(y, s), PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))


def _spd(D, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((D, D))
    return (A @ A.T / D + 0.5 * np.eye(D)).astype(np.float32)


@pytest.mark.gpu
def test_dense_init_factorisation_matches_oracle():
    model, _ = _hier()
    D = model.latent_dim
    A = _spd(D)
    k = NUTS(model, num_chains=4, dense_mass=True, inverse_mass_matrix=A)
    st = k.init(SEED, 0)
    a = st.adapt_state
    inv, sq, sqi = R._initialize_mass_matrix(D, A.astype(np.float64), True)
    for c in range(4):
        np.testing.assert_array_equal(a.inverse_mass_matrix[c].cpu().numpy(), A)
        np.testing.assert_allclose(a.mass_matrix_sqrt[c].cpu().numpy(), sq, rtol=2e-5, atol=2e-6)
        np.testing.assert_allclose(a.mass_matrix_sqrt_inv[c].cpu().numpy(), sqi, rtol=2e-5, atol=2e-6)
    # M^-1 = T^T T and M = S S^T
    T, S = a.mass_matrix_sqrt_inv[0].double().cpu().numpy(), a.mass_matrix_sqrt[0].double().cpu().numpy()
    np.testing.assert_allclose(T.T @ T, A, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(S @ S.T @ A, np.eye(D), atol=1e-4)
    k.close()


@pytest.mark.gpu
def test_dense_single_transition_parity():
    model, pot = _hier()
    D = model.latent_dim
    A = _spd(D, seed=1)
    C = 128
    k = NUTS(model, num_chains=C, step_size=0.3, adapt_step_size=False, adapt_mass_matrix=False, dense_mass=True,
             inverse_mass_matrix=A)
    state = k.init(SEED, 0)
    steps = [0.05, 0.2, 0.5, 1.0]
    state.adapt_state.step_size.copy_(torch.tensor([steps[c % 4] for c in range(C)], dtype=torch.float32,
                                                   device="cuda"))
    same, total, zerr = 0, 0, []
    for it in range(4):
        z0 = state.z.cpu().numpy().copy()
        new = k.sample(state)
        zg, ns, dv = new.z.cpu().numpy(), new.num_steps.cpu().numpy(), new.diverging.cpu().numpy()
        for c in range(C):
            init_kernel, sample_kernel = R.hmc(pot)
            ost = init_kernel(z0[c].astype(np.float64), 0, step_size=steps[c % 4],
                              inverse_mass_matrix=A.astype(np.float64), adapt_step_size=False,
                              adapt_mass_matrix=False, dense_mass=True, rng_key=(SEED, c))
            ref = sample_kernel(ost._replace(rng_key=R.RngKey(SEED, c, it)))
            total += 1
            if ref.num_steps == ns[c] and bool(ref.diverging) == bool(dv[c]):
                same += 1
                zerr.append(np.max(np.abs(ref.z - zg[c]) / (np.abs(ref.z) + 1e-2)))
        state = new
    assert same / total >= 0.99, same / total
    assert np.median(zerr) < 1e-5, np.median(zerr)
    k.close()


@pytest.mark.gpu
def test_dense_welford_window_end_matches_oracle():
    """Stage Welford accumulators at the end of the first middle window; one transition later the
    device's mass matrices equal the oracle's update_fn + final_fn(regularize=True) on that draw."""
    model, _ = _hier()
    D = model.latent_dim
    C, W = 8, 200
    sched = R.build_adaptation_schedule(W)
    t_end = sched[1].end  # last iteration of the first slow window
    k = NUTS(model, num_chains=C, dense_mass=True)
    st = k.init(SEED, W)
    rng = np.random.default_rng(3)
    n0 = sched[1].end - sched[1].start  # draws already accumulated in the window
    mean0 = rng.standard_normal((C, D))
    X = rng.standard_normal((C, n0, D)) @ np.linalg.cholesky(_spd(D, 2).astype(np.float64)).T
    m20 = np.einsum("cni,cnj->cij", X - X.mean(1, keepdims=True), X - X.mean(1, keepdims=True))
    a = st.adapt_state
    st.i.fill_(t_end)
    a.window_idx.fill_(1)
    a.mm_state[0].copy_(torch.as_tensor(mean0, device="cuda"))
    a.mm_state[1].copy_(torch.as_tensor(m20, device="cuda"))
    a.mm_state[2].fill_(n0)
    new = k.sample(st)
    zn = new.z.double().cpu().numpy()
    init_fn, update_fn, final_fn = R.welford_covariance(diagonal=False)
    na = new.adapt_state
    for c in range(C):
        mm = update_fn(zn[c], (mean0[c], m20[c], n0))
        cov, sq, sqi = final_fn(mm, regularize=True)
        np.testing.assert_allclose(na.inverse_mass_matrix[c].cpu().numpy(), cov, rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(na.mass_matrix_sqrt[c].cpu().numpy(), sq, rtol=2e-5, atol=2e-6)
        np.testing.assert_allclose(na.mass_matrix_sqrt_inv[c].cpu().numpy(), sqi, rtol=2e-5, atol=2e-6)
    assert int(na.mm_state[2].max()) == 0 and float(na.mm_state[1].abs().max()) == 0.0
    assert np.all(na.window_idx.cpu().numpy() == 2)
    k.close()


@pytest.mark.gpu
def test_dense_mass_mcmc_matches_diagonal_posterior():
    model, _ = _hier()
    res = {}
    for dense in (False, True):
        mcmc = MCMC(NUTS(model, dense_mass=dense), num_warmup=400, num_samples=600, num_chains=16)
        mcmc.run(7)
        res[dense] = mcmc.get_samples(group_by_chain=True)
    for site in ("mu", "tau"):
        a, b = res[True][site].reshape(16, 600, -1), res[False][site].reshape(16, 600, -1)
        m1, m2 = a.mean(axis=(0, 1)), b.mean(axis=(0, 1))
        e1 = np.array([diagnostics.effective_sample_size(a[..., d]) for d in range(a.shape[-1])])
        e2 = np.array([diagnostics.effective_sample_size(b[..., d]) for d in range(b.shape[-1])])
        mcse = np.sqrt(a.std(axis=(0, 1)) ** 2 / e1 + b.std(axis=(0, 1)) ** 2 / e2)
        assert np.all(np.abs(m1 - m2) <= 4 * mcse), (site, m1, m2, mcse)
        assert np.all(diagnostics.split_gelman_rubin(a) < 1.05)


@pytest.mark.gpu
def test_block_structured_window_end_matches_numpyro_blocks():
    """dense_mass=[("theta_base", "mu")] (numpyro's list form, hmc_util.py:439-486): one dense block
    over theta_base and mu -- listed out of the sites' order, with tau between them in z -- and
    tau in the remaining diagonal block.  At the window end the device's inverse mass matrix is
    the oracle's welford final_fn of each block (dense for the tuple, diagonal for the rest) in
    the full coordinates and zero across blocks, and its square roots reproduce M^-1 and M."""
    model, _ = _hier()
    D = model.latent_dim
    sl = model.site_slices()
    blockA = list(range(*sl["theta_base"][:2])) + list(range(*sl["mu"][:2]))  # the tuple's order
    diag = list(range(*sl["tau"][:2]))
    C, W = 8, 200
    sched = R.build_adaptation_schedule(W)
    t_end = sched[1].end
    k = NUTS(model, num_chains=C, dense_mass=[("theta_base", "mu")])
    st = k.init(SEED, W)
    rng = np.random.default_rng(5)
    n0 = sched[1].end - sched[1].start
    mean0 = rng.standard_normal((C, D))
    X = rng.standard_normal((C, n0, D)) @ np.linalg.cholesky(_spd(D, 3).astype(np.float64)).T
    m20 = np.einsum("cni,cnj->cij", X - X.mean(1, keepdims=True), X - X.mean(1, keepdims=True))
    a = st.adapt_state
    st.i.fill_(t_end)
    a.window_idx.fill_(1)
    a.mm_state[0].copy_(torch.as_tensor(mean0, device="cuda"))
    a.mm_state[1].copy_(torch.as_tensor(m20, device="cuda"))
    a.mm_state[2].fill_(n0)
    new = k.sample(st)
    zn = new.z.double().cpu().numpy()
    na = new.adapt_state
    _, upd_d, fin_d = R.welford_covariance(diagonal=False)
    _, upd_v, fin_v = R.welford_covariance(diagonal=True)
    for c in range(C):
        inv = na.inverse_mass_matrix[c].double().cpu().numpy()
        sq = na.mass_matrix_sqrt[c].double().cpu().numpy()
        sqi = na.mass_matrix_sqrt_inv[c].double().cpu().numpy()
        ia = np.ix_(blockA, blockA)
        mm = upd_d(zn[c][blockA], (mean0[c][blockA], m20[c][ia], n0))
        covA, _, _ = fin_d(mm, regularize=True)
        mv = upd_v(zn[c][diag], (mean0[c][diag], np.diag(m20[c])[diag], n0))
        varD, _, _ = fin_v(mv, regularize=True)
        expect = np.zeros((D, D))
        expect[ia] = covA
        expect[diag, diag] = varD
        np.testing.assert_allclose(inv, expect, rtol=1e-5, atol=1e-7)
        # numpyro's factors: mass_matrix_sqrt_inv^T mass_matrix_sqrt_inv = M^-1, sqrt sqrt^T = M
        np.testing.assert_allclose(sqi.T @ sqi, expect, rtol=2e-5, atol=2e-6)
        np.testing.assert_allclose(sq @ sq.T, np.linalg.inv(expect), rtol=2e-4, atol=2e-5)
        assert np.all(sq[np.ix_(diag, blockA)] == 0) and np.all(sq[np.ix_(blockA, diag)] == 0)
    k.close()


@pytest.mark.gpu
def test_block_structured_mass_mcmc_matches_diagonal_posterior():
    model, _ = _hier()
    res = {}
    for dense in (False, [("mu", "tau")]):
        mcmc = MCMC(NUTS(model, dense_mass=dense), num_warmup=400, num_samples=600, num_chains=16)
        mcmc.run(8)
        res[bool(dense)] = mcmc.get_samples(group_by_chain=True)
    for site in ("mu", "tau"):
        a, b = res[True][site].reshape(16, 600, -1), res[False][site].reshape(16, 600, -1)
        m1, m2 = a.mean(axis=(0, 1)), b.mean(axis=(0, 1))
        mcse = np.sqrt(diagnostics.mcse_mean(a) ** 2 + diagnostics.mcse_mean(b) ** 2)
        assert np.all(np.abs(m1 - m2) <= 4 * mcse), (site, m1, m2, mcse)
        assert np.all(diagnostics.split_gelman_rubin(a) < 1.05)
