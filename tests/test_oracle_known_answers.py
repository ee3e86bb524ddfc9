"""Pins the FP64 oracle against the known answers of numpyro's own tests.

Each test restates a test of numpyro's test suite (file:line cited) against
``oracle/nuts_ref.py``; numpyro itself cannot run here (no jax), so these
known answers are what ties the restatement to the reference.
"""
import math

import numpy as np
from numpy.testing import assert_allclose
import pytest

from oracle import nuts_ref as R
from oracle import philox


def test_philox_known_answer_vectors():
    # Random123 kat_vectors for philox4x32-10 (Salmon et al. 2011)
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, expect in cases:
        out = philox.philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32))
        assert tuple(int(x) for x in out) == expect


def test_philox_normals_moments():
    z = np.concatenate([philox.normals(7, c, 0, philox.MOMENTUM, 1000) for c in range(50)])
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1) < 0.02


def test_dual_averaging():
    # test/infer/test_hmc_util.py:36-52: minimise (x+1)^2 with gamma=0.5
    da_init, da_update = R.dual_averaging(gamma=0.5)
    state = da_init()
    for _ in range(10):
        x = state[0]
        g = 2 * (x + 1)
        state = da_update(g, state)
    assert_allclose(state[1], -1.0, atol=1e-3)


@pytest.mark.parametrize("diagonal", [True, False])
@pytest.mark.parametrize("regularize", [True, False])
def test_welford_covariance(diagonal, regularize):
    # test/infer/test_hmc_util.py:55-89
    rng = np.random.RandomState(0)
    loc = rng.randn(3)
    a = rng.randn(3, 3)
    target_cov = a @ a.T
    x = rng.multivariate_normal(loc, target_cov, size=(2000,))
    wc_init, wc_update, wc_final = R.welford_covariance(diagonal=diagonal)
    st = wc_init(3)
    for i in range(2000):
        st = wc_update(x[i], st)
    cov, cov_inv_sqrt, _ = wc_final(st, regularize=regularize)
    if diagonal:
        diag_cov = np.diagonal(target_cov)
        assert_allclose(cov, diag_cov, rtol=0.06)
        assert_allclose(cov_inv_sqrt, np.sqrt(np.reciprocal(diag_cov)), rtol=0.06)
    else:
        assert_allclose(cov, target_cov, rtol=0.06)
        assert_allclose(cov_inv_sqrt, np.linalg.cholesky(np.linalg.inv(cov)), rtol=0.06)


# test/infer/test_hmc_util.py:121-191: analytic oscillators
def _harmonic(q):
    return 0.5 * float(q @ q), q.copy()


def _planetary(q):
    rr = math.sqrt(q[0] ** 2 + q[1] ** 2)
    return -1.0 / rr, q / rr ** 3


def _quartic(q):
    return 0.25 * float(np.sum(q ** 4)), q ** 3


OSCILLATORS = [
    (_harmonic, 0.01, 100, [0.0], [1.0], [math.sin(1.0)], [math.cos(1.0)], [1.0], 1e-4),
    (_planetary, 0.01, 628, [1.0, 0.0], [0.0, 1.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], 5e-3),
    (_quartic, 0.1, 1810, [0.02], [0.0], [-0.02], [0.0], [1.0], 1e-4),
]


@pytest.mark.parametrize("case", OSCILLATORS, ids=["harmonic", "planetary", "quartic"])
def test_velocity_verlet(case):
    # test/infer/test_hmc_util.py:194-229
    pot, step, nsteps, qi, pi, qf, pf, minv, prec = case
    m_inv = np.array(minv)
    vv_init, vv_update = R.velocity_verlet(pot)

    def run(q, p):
        st = vv_init(np.array(q, float), np.array(p, float))
        for _ in range(nsteps):
            st = vv_update(step, m_inv, st)
        return st

    st = run(qi, pi)
    assert_allclose(st.z, qf, atol=prec)
    assert_allclose(st.r, pf, atol=prec)
    e0 = R.euclidean_kinetic_energy(m_inv, np.array(pi, float)) + pot(np.array(qi, float))[0]
    e1 = R.euclidean_kinetic_energy(m_inv, st.r) + st.potential_energy
    assert_allclose(e0, e1, atol=1e-5)
    back = run(st.z, -st.r)
    assert_allclose(back.z, qi, atol=1e-4)


@pytest.mark.parametrize("init_step_size", [0.1, 10.0])
def test_find_reasonable_step_size(init_step_size):
    # test/infer/test_hmc_util.py:232-275 (momentum stubbed to 1.0)
    def pot(q):
        return 0.5 * float(q[0] ** 2), np.array([q[0]])

    m_inv = np.array([1.0])
    step = R.find_reasonable_step_size(pot, R.euclidean_kinetic_energy, init_step_size, m_inv,
                                       (np.array([0.0]), None, None, None), R.RngKey(0, 0, 0),
                                       momentum_fn=lambda m: np.array([1.0]))
    threshold = (-math.log(0.8) * 8) ** 0.25
    if init_step_size < threshold:
        assert step / 2 < threshold
        assert step > threshold
    else:
        assert step * 2 > threshold
        assert step < threshold


@pytest.mark.parametrize(
    "num_steps, expected",
    [
        (18, [(0, 17)]),
        (50, [(0, 6), (7, 44), (45, 49)]),
        (100, [(0, 14), (15, 89), (90, 99)]),
        (150, [(0, 74), (75, 99), (100, 149)]),
        (200, [(0, 74), (75, 99), (100, 149), (150, 199)]),
        (280, [(0, 74), (75, 99), (100, 229), (230, 279)]),
    ],
)
def test_build_adaptation_schedule(num_steps, expected):
    # test/infer/test_hmc_util.py:278-292 (exact table)
    assert R.build_adaptation_schedule(num_steps) == [R.AdaptWindow(i, j) for i, j in expected]


def test_warmup_adapter():
    # test/infer/test_hmc_util.py:295-378
    def frs(step_size, m_inv, z, rng_key):
        return step_size * 4 if step_size < 1 else step_size / 4

    num_steps = 150
    sched = R.build_adaptation_schedule(num_steps)
    wa_init, wa_update = R.warmup_adapter(num_steps, frs)
    z = np.ones(3)
    st = wa_init((z, None, None, None), R.RngKey(0, 0, 0), 1.0, mass_matrix_size=3)
    assert st.step_size == frs(1.0, None, None, None)
    assert_allclose(st.inverse_mass_matrix, np.ones(3))
    assert st.window_idx == 0

    w = sched[0]
    for t in range(w.start, w.end + 1):
        st = wa_update(t, 0.7 + 0.1 * t / (w.end - w.start), (z,), st)
    last = frs(1.0, None, None, None)
    assert st.window_idx == 1
    assert st.step_size < last
    assert_allclose(st.inverse_mass_matrix, np.ones(3))

    w = sched[1]
    wl = w.end - w.start
    last = st.step_size
    for t in range(w.start, w.end + 1):
        st = wa_update(t, 0.8 + 0.1 * (t - w.start) / wl, (2 * z,), st)
    assert st.window_idx == 2
    assert st.step_size > last
    reg = 1e-3 * (5 / (w.end + 1 - w.start + 5))
    assert_allclose(st.inverse_mass_matrix, np.full(3, reg), atol=1e-7)
    inv_mass = st.inverse_mass_matrix

    w = sched[2]
    last = st.step_size
    for t in range(w.start, w.end + 1):
        st = wa_update(t, 0.8, (t * z,), st)
    assert st.window_idx == 3
    assert_allclose(st.step_size, last * 10, atol=1e-6)
    assert_allclose(st.inverse_mass_matrix, inv_mass)


@pytest.mark.parametrize("leaf_idx, ckpt_idxs", [(0, (1, 0)), (6, (3, 2)), (7, (0, 2)), (13, (2, 2)), (15, (0, 3))])
def test_leaf_idx_to_ckpt_idx(leaf_idx, ckpt_idxs):
    # test/infer/test_hmc_util.py:381-386 (exact table)
    assert R.leaf_idx_to_ckpt_idxs(leaf_idx) == ckpt_idxs


@pytest.mark.parametrize(
    "ckpt_idxs, expected_turning",
    [((3, 2), False), ((3, 3), True), ((0, 0), False), ((0, 1), True), ((1, 3), True)],
)
def test_is_iterative_turning(ckpt_idxs, expected_turning):
    # test/infer/test_hmc_util.py:389-403 (exact truth table)
    r_ckpts = np.array([[1.0], [2.0], [3.0], [-2.0]])
    r_sum_ckpts = np.array([[2.0], [4.0], [4.0], [-1.0]])
    got = R.is_iterative_turning(np.ones(1), np.array([1.0]), np.array([3.0]), r_ckpts, r_sum_ckpts, *ckpt_idxs)
    assert got == expected_turning


@pytest.mark.parametrize("step_size", [0.01, 1.0, 100.0])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_build_tree(step_size, seed):
    # test/infer/test_hmc_util.py:406-442 (invariants)
    def pot(q):
        return 0.5 * float(q[0] ** 2), np.array([q[0]])

    vv_init, vv_update = R.velocity_verlet(pot)
    st = vv_init(np.array([0.0]), np.array([1.0]))
    tree = R.build_tree(vv_update, R.euclidean_kinetic_energy, st, np.array([1.0]), step_size,
                        R.RngKey(seed, 0, 0))
    assert tree.num_proposals >= 2 ** (tree.depth - 1)
    assert tree.sum_accept_probs <= tree.num_proposals
    if tree.depth < 10:
        assert tree.turning or tree.diverging
    if step_size > 10:
        assert tree.diverging
        assert tree.num_proposals == 1
    if step_size < 0.1:
        assert tree.num_proposals > 10


def test_masked_dense_welford_is_numpyros_block_structured_mass():
    """The engine's block-structured mass (dense Welford over all coordinates, then only in-block
    entries and the diagonal kept) equals numpyro's per-block adaptation (hmc_util.py:439-486: a
    dense welford_covariance per listed block, a diagonal one for the rest), and the reverse
    Cholesky factors of that block-diagonal matrix have no fill-in, with blocks interleaved in the
    coordinates and a block listed out of coordinate order."""
    rng = np.random.RandomState(1)
    D, n = 7, 400
    a = rng.randn(D, D)
    x = rng.multivariate_normal(rng.randn(D), a @ a.T + np.eye(D), size=n)
    blocks = [[5, 1, 3], [0, 6]]  # tuple order as listed; coordinates 2 and 4 in the diagonal block
    rest = [2, 4]
    full = R.welford_covariance(diagonal=False)
    st = full[0](D)
    for i in range(n):
        st = full[1](x[i], st)
    cov_full, _, _ = full[2](st, regularize=True)
    keep = np.eye(D, dtype=bool)
    for b in blocks:
        keep[np.ix_(b, b)] = True
    masked = np.where(keep, cov_full, 0.0)
    expect = np.zeros((D, D))
    for b in blocks:
        dense = R.welford_covariance(diagonal=False)
        sb = dense[0](len(b))
        for i in range(n):
            sb = dense[1](x[i][b], sb)
        expect[np.ix_(b, b)], _, _ = dense[2](sb, regularize=True)
    diag = R.welford_covariance(diagonal=True)
    sd = diag[0](len(rest))
    for i in range(n):
        sd = diag[1](x[i][rest], sd)
    expect[rest, rest], _, _ = diag[2](sd, regularize=True)
    assert_allclose(masked, expect, rtol=1e-12, atol=1e-14)
    # the factors final_fn forms from a covariance equal to the masked matrix (m2 = cov (n - 1))
    _, sq, sqi = full[2]((np.zeros(D), masked * (n - 1), n), regularize=False)
    assert np.all(sq[~keep] == 0.0) and np.all(sqi[~keep] == 0.0)
    assert_allclose(sqi.T @ sqi, masked, rtol=1e-10, atol=1e-12)
    assert_allclose(sq @ sq.T, np.linalg.inv(masked), rtol=1e-9, atol=1e-10)
