"""Generates the golden fixtures of tests/golden/ from the FP64 oracle.

numpyro itself cannot be imported here (it needs jax), so these fixtures come
from the oracle restatement, which is pinned to numpyro's own known answers
(tests/test_oracle_known_answers.py).  They freeze the oracle's NUTS behaviour on
the injected Philox stream so that later changes to the oracle, and the GPU
parity tests, compare against fixed numbers.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from numpyro_gb300 import datasets  # noqa: E402
from oracle import nuts_ref as R  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402

SEED = 20261203


def main():
    y, s = datasets.eight_schools(0)
    pot = PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))
    C, T = 6, 12
    z0 = np.stack([R.init_to_uniform(SEED, c, 10) for c in range(C)])
    traj = np.zeros((C, T, 10))
    steps = np.zeros((C, T), np.int64)
    acc = np.zeros((C, T))
    step_size = np.zeros((C, T))
    for c in range(C):
        init_kernel, sample_kernel = R.hmc(pot)
        st = init_kernel(z0[c], 50, rng_key=(SEED, c))
        for t in range(T):
            st = sample_kernel(st)
            traj[c, t] = st.z
            steps[c, t] = st.num_steps
            acc[c, t] = st.accept_prob
            step_size[c, t] = st.adapt_state.step_size
    np.savez_compressed(os.path.join(HERE, "nuts_hier_nc_warmup.npz"), seed=SEED, z0=z0, z=traj, num_steps=steps,
                        accept_prob=acc, step_size=step_size, y=y, sigma=s)
    # potentials at fixed points, one file per family
    rng = np.random.default_rng(SEED)
    X, yy, _ = datasets.covtype_like(seed=7, n=400, n_cont=3, n_bin=3)
    zl = 0.3 * rng.standard_normal((4, X.shape[1]))
    pe = np.array([PR.logreg_potential(z, X.astype(np.float64), yy.astype(np.float64)) for z in zl])
    g = np.stack([PR.logreg_grad(z, X.astype(np.float64), yy.astype(np.float64)) for z in zl])
    np.savez_compressed(os.path.join(HERE, "potential_logreg.npz"), X=X, y=yy, z=zl, pe=pe, grad=g)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
