"""The C oracle (timed CPU baseline) agrees with the FP64 Python restatement."""
import numpy as np
import pytest

from numpyro_gb300 import datasets
from oracle import build_oracle as B
from oracle import nuts_ref as R
from oracle import potentials_ref as PR


@pytest.fixture(scope="module")
def lib64():
    return B.load("f64")


def test_fixed_step_trajectories_match(lib64):
    y, s = datasets.eight_schools(0)
    pot = PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))
    res = B.run_hier(lib64, y, s, chains=3, num_warmup=0, num_samples=25, seed=5, threads=2)
    for c in range(3):
        sp, ex, _ = R.run_chain(pot, 10, 5, c, 0, 25)
        np.testing.assert_array_equal(ex["num_steps"], res["num_steps"][c])
        np.testing.assert_allclose(res["samples"][c], sp, rtol=1e-6, atol=1e-6)


def test_warmup_adaptation_matches_initially(lib64):
    """Dual averaging + windows: identical draws until ulp differences grow (chaos)."""
    y, s = datasets.eight_schools(0)
    pot = PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))
    res = B.run_hier(lib64, y, s, chains=2, num_warmup=20, num_samples=12, seed=9, threads=2)
    for c in range(2):
        sp, ex, _ = R.run_chain(pot, 10, 9, c, 20, 12)
        assert (ex["num_steps"] == res["num_steps"][c]).mean() >= 0.75


def test_logreg_c_oracle_fixed_step(lib64):
    X, y, beta = datasets.covtype_like(seed=2, n=500, n_cont=2, n_bin=2)
    pot = PR.make_potential("logreg", X.astype(np.float64), y.astype(np.float64))
    D = X.shape[1]
    z0 = np.tile(beta.astype(np.float32), (2, 1))
    init = (z0, np.full(2, 0.1, np.float32), np.ones((2, D), np.float32))
    res = B.run_logreg(lib64, X, y, chains=2, num_warmup=0, num_samples=10, seed=3, threads=2, init=init)
    for c in range(2):
        init_kernel, sample_kernel = R.hmc(pot)
        st = init_kernel(z0[c].astype(np.float64), 0, step_size=0.1, rng_key=(3, c))
        steps = []
        for _ in range(10):
            st = sample_kernel(st)
            steps.append(st.num_steps)
        np.testing.assert_array_equal(steps, res["num_steps"][c])
        np.testing.assert_allclose(res["samples"][c][-1], st.z, rtol=1e-5, atol=1e-6)


def _family_cases():
    from gpu_helpers import typical_points  # noqa: F401  (plain numpy helper)

    y, s = datasets.eight_schools(0)
    X, yy, _ = datasets.covtype_like(seed=1, n=3000, n_cont=4, n_bin=6)
    Xh, yh, _ = datasets.horseshoe_data(seed=2, n=200, p=50, nonzero=5)
    r, _ = datasets.sv_returns(seed=3, T=300)
    f64 = lambda a: a.astype(np.float64)  # noqa: E731
    return [
        ("hier_nc", B.Model("hier_nc", y=y, sigma=s), (f64(y), f64(s)), 10, 0.3),
        ("logreg", B.Model("logreg", X=X, y=yy), (f64(X), f64(yy)), X.shape[1], 0.02),
        ("horseshoe", B.Model("horseshoe", X=Xh, y=yh), (f64(Xh), f64(yh)), 102, 0.01),
        ("horseshoe_nc", B.Model("horseshoe_nc", X=Xh, y=yh), (f64(Xh), f64(yh)), 102, 0.02),
        ("sv", B.Model("sv", y=r), (f64(r),), 302, 0.005),
        ("sv_nc", B.Model("sv_nc", y=r), (f64(r),), 302, 0.01),
    ]


class _Dim:
    def __init__(self, d):
        self.latent_dim = d


def test_c_potentials_match_python_restatement(lib64):
    """Every family's C potential and gradient equal the FP64 Python restatement (itself pinned
    to scipy.stats and central differences in test_oracle_potentials.py)."""
    from gpu_helpers import typical_points

    rng = np.random.default_rng(0)
    for name, m, data, D, _ in _family_cases():
        assert lib64.nutsref_latent_dim(m.ref(), 0) == D
        z = typical_points(name, _Dim(D), rng, 3).astype(np.float64)
        pot, grad = PR.FAMILIES[name]
        for c in range(3):
            pe, g = B.potential(lib64, m, z[c])
            pr, gr = pot(z[c], *data), grad(z[c], *data)
            assert abs(pe - pr) <= 1e-12 * abs(pr), (name, pe, pr)
            np.testing.assert_allclose(g, gr, rtol=1e-10, atol=1e-10 * np.abs(gr).max(), err_msg=name)


def test_c_uneven_hierarchical_models_follow_chain_ids(lib64):
    ds = datasets.uneven_hierarchical(seed=1, num_models=5, jmin=3, jmax=30)
    y = np.concatenate([a for a, _ in ds])
    s = np.concatenate([b for _, b in ds])
    off = np.zeros(6, np.int32)
    off[1:] = np.cumsum([len(a) for a, _ in ds])
    m = B.Model("hier_nc", y=y, sigma=s, offsets=off, chains_per_model=3)
    rng = np.random.default_rng(1)
    for k, (yk, sk) in enumerate(ds):
        D = len(yk) + 2
        assert lib64.nutsref_latent_dim(m.ref(), k) == D
        z = rng.uniform(-2, 2, D)
        pe, g = B.potential(lib64, m, z, model_index=k)
        assert abs(pe - PR.hier_nc_potential(z, f64(yk), f64(sk))) < 1e-10 * abs(pe)
        np.testing.assert_allclose(g, PR.hier_nc_grad(z, f64(yk), f64(sk)), rtol=1e-10, atol=1e-12)
    # one transition of chain 7 (dataset 7 // 3 = 2) equals the oracle on dataset 2 alone
    D2 = len(ds[2][0]) + 2
    ld = max(len(a) for a, _ in ds) + 2
    z0 = np.zeros((1, ld), np.float32)
    z0[0, :D2] = rng.uniform(-1, 1, D2)
    out = B.transitions(lib64, m, z0, 0.2, np.ones(ld), np.ones(ld), 7, 0, 11)
    pot = PR.make_potential("hier_nc", f64(ds[2][0]), f64(ds[2][1]))
    init_kernel, sample_kernel = R.hmc(pot)
    st = init_kernel(z0[0, :D2].astype(np.float64), 0, step_size=float(np.float32(0.2)), rng_key=(11, 7))
    st = sample_kernel(st)
    assert st.num_steps == out["num_steps"][0]
    np.testing.assert_allclose(out["z"][0, :D2], st.z, rtol=1e-6, atol=1e-7)
    assert np.all(out["z"][0, D2:] == 0)


def f64(a):
    return np.asarray(a, np.float64)


def test_c_transitions_match_python_restatement(lib64):
    """One NUTS transition per chain from given states: identical tree sizes, divergences and
    accept probabilities, positions to FP64 rounding (stored as float32)."""
    from gpu_helpers import typical_points

    rng = np.random.default_rng(0)
    seed = 77
    for name, m, data, D, step in _family_cases():
        C = 4
        z = typical_points(name, _Dim(D), rng, C)
        inv = rng.uniform(0.5, 2.0, (C, D)).astype(np.float32)
        msq = (1.0 / np.sqrt(inv)).astype(np.float32)
        out = B.transitions(lib64, m, z, step, inv, msq, np.arange(C), 3, seed)
        pot = PR.make_potential(name, *data)
        for c in range(C):
            init_kernel, sample_kernel = R.hmc(pot)
            st = init_kernel(z[c].astype(np.float64), 0, step_size=float(np.float32(step)),
                             inverse_mass_matrix=inv[c].astype(np.float64), adapt_step_size=False,
                             adapt_mass_matrix=False, rng_key=(seed, c))
            st = sample_kernel(st._replace(rng_key=R.RngKey(seed, c, 3)))
            assert st.num_steps == out["num_steps"][c], (name, c)
            assert bool(st.diverging) == bool(out["diverging"][c]), (name, c)
            assert abs(st.accept_prob - out["accept_prob"][c]) < 1e-7, (name, c)
            np.testing.assert_allclose(out["z"][c], st.z, rtol=2e-6, atol=1e-6, err_msg="%s %d" % (name, c))


def test_f32_build_potentials_match_f64():
    """The FP32 build (numpyro's float32 dtype; the timed CPU baseline, with its own vectorisable
    exp and log1p for the logistic rows) agrees with the FP64 build to FP32 rounding."""
    from gpu_helpers import typical_points

    lib32, lib64 = B.load("f32"), B.load("f64")
    rng = np.random.default_rng(3)
    X, yy, beta = datasets.covtype_like(seed=0, n=20000)
    m = B.Model("logreg", X=X, y=yy)
    for sc in (0.01, 1.0, 5.0):
        z = beta + sc * rng.standard_normal(beta.shape)
        p64, g64 = B.potential(lib64, m, z)
        p32, g32 = B.potential(lib32, m, z)
        assert abs(p32 - p64) <= 1e-6 * abs(p64), (sc, p32, p64)
        assert np.max(np.abs(g32 - g64)) <= 1e-5 * np.max(np.abs(g64)), sc
    for name, mm, _, D, _ in _family_cases():
        z = typical_points(name, _Dim(D), rng, 2).astype(np.float64)
        for c in range(2):
            p64, g64 = B.potential(lib64, mm, z[c])
            p32, g32 = B.potential(lib32, mm, z[c])
            assert abs(p32 - p64) <= 1e-5 * abs(p64) + 1e-4, (name, p32, p64)
            assert np.max(np.abs(g32 - g64)) <= 1e-4 * np.max(np.abs(g64)) + 1e-4, name
