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
