"""NUTS/HMC transition parity: CUDA engine vs the FP64 oracle on identical Philox bits.

Each GPU transition is replayed by the oracle from the GPU's own starting
state (so FP32-vs-FP64 chaos cannot accumulate), with the same stream
addresses.  Tree sizes (num_steps) must agree on >= 99.9% of transitions,
positions within 1e-5 relative (median) on trajectories that take the same decisions.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import HMC, NUTS, datasets, models  # noqa: E402
from oracle import nuts_ref as R  # noqa: E402
from oracle import philox  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402

SEED = 1234


def _hier():
    y, s = datasets.eight_schools(0)
    return models.HierarchicalNormal(y, s), PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))


def _oracle_transition(pot, z, step, inv_mass, chain, n, algo="NUTS", max_tree_depth=10, traj=None, nsteps=None):
    init_kernel, sample_kernel = R.hmc(pot, algo=algo)
    kw = {}
    if algo == "HMC":
        kw = dict(trajectory_length=traj, num_steps=nsteps)
    st = init_kernel(np.asarray(z, np.float64), 0, step_size=step, inverse_mass_matrix=np.asarray(inv_mass, np.float64),
                     adapt_step_size=False, adapt_mass_matrix=False, max_tree_depth=max_tree_depth,
                     rng_key=(SEED, chain), **kw)
    st = st._replace(rng_key=R.RngKey(SEED, chain, n))
    return sample_kernel(st)


@pytest.mark.gpu
def test_init_to_uniform_bits_match_oracle():
    model, _ = _hier()
    C = 64
    k = NUTS(model, num_chains=C)
    st = k.init(SEED, 0)
    z = st.z.cpu().numpy()
    for c in range(C):
        np.testing.assert_array_equal(z[c], R.init_to_uniform(SEED, c, model.latent_dim).astype(np.float32))
    k.close()


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ["fused", "plain"])
def test_single_transition_parity(engine):
    model, pot = _hier()
    C = 256
    steps = [0.05, 0.2, 0.6, 1.5]
    k = NUTS(model, num_chains=C, step_size=0.3, adapt_step_size=False, adapt_mass_matrix=False, engine=engine)
    state = k.init(SEED, 0)
    # per-chain step sizes and masses to exercise deep trees, U-turns and divergences
    ss = torch.tensor([steps[c % 4] for c in range(C)], dtype=torch.float32, device="cuda")
    inv = torch.as_tensor(np.random.default_rng(0).uniform(0.5, 2.0, (C, model.latent_dim)).astype(np.float32),
                          device="cuda")
    state.adapt_state.step_size.copy_(ss)
    state.adapt_state.inverse_mass_matrix.copy_(inv)
    state.adapt_state.mass_matrix_sqrt.copy_(1.0 / inv.sqrt())
    same, total, zerr = 0, 0, []
    for it in range(8):
        z0 = state.z.cpu().numpy().copy()
        new = k.sample(state)
        zg = new.z.cpu().numpy()
        ns = new.num_steps.cpu().numpy()
        ap = new.accept_prob.cpu().numpy()
        dv = new.diverging.cpu().numpy()
        for c in range(C):
            ref = _oracle_transition(pot, z0[c], steps[c % 4], inv[c].cpu().numpy(), c, it)
            total += 1
            if ref.num_steps == ns[c] and bool(ref.diverging) == bool(dv[c]):
                same += 1
                assert abs(ref.accept_prob - ap[c]) <= 1e-3 + 1e-3 * abs(ref.accept_prob)
                zerr.append(np.max(np.abs(ref.z - zg[c]) / (np.abs(ref.z) + 1e-2)))
        state = new
    frac = same / total
    print("tree sizes identical on %d of %d transitions (%.4f)" % (same, total, frac))
    assert frac >= 0.999, frac  # 2048 transitions: at most 2 may part
    assert np.median(zerr) < 1e-5, np.median(zerr)
    k.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["hier", "uneven", "sv", "sv_nc"])
def test_persistent_tick_and_plain_engines_are_bit_identical(case):
    """The persistent launch (fused), the launch-per-leapfrog tick engine and the lock-step
    plain engine take identical decisions on identical bits: draws, tree sizes and adapted
    step sizes agree bit for bit.  The hierarchical family runs a warp per chain, the
    stochastic-volatility family a CTA per chain."""
    iters = 150
    if case == "uneven":
        model = models.HierarchicalNormal(datasets=datasets.uneven_hierarchical(seed=1, num_models=9, jmin=3,
                                                                                 jmax=40))
        C = 36
    elif case in ("sv", "sv_nc"):
        r, _ = datasets.sv_returns(seed=2, T=300)
        model = models.StochasticVolatility(r, noncentered=(case == "sv_nc"))
        C, iters = 8, 60
    else:
        model, _ = _hier()
        C = 32
    res = {}
    for engine in ["fused", "ticks", "plain"]:
        k = NUTS(model, num_chains=C, engine=engine, max_tree_depth=8)
        st = k.init(SEED, iters // 2)
        out = k.run_device(st, iters, collect_start=0, collect=("z", "num_steps"))
        res[engine] = (out["z"].cpu().numpy(), out["num_steps"].cpu().numpy(), st.adapt_state.step_size.cpu().numpy())
        k.close()
    for a, b, c in zip(res["fused"], res["ticks"], res["plain"]):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)


@pytest.mark.gpu
def test_warmup_adaptation_tracks_oracle():
    """First iterations of warmup (dual averaging) follow the oracle's step-size sequence."""
    model, pot = _hier()
    C = 8
    k = NUTS(model, num_chains=C)
    st = k.init(SEED, 50)
    gpu_steps = []
    for it in range(8):
        st = k.sample(st)
        gpu_steps.append(st.adapt_state.step_size.cpu().numpy().copy())
    gpu_steps = np.array(gpu_steps)
    agree = 0
    for c in range(C):
        init_kernel, sample_kernel = R.hmc(pot)
        ost = init_kernel(R.init_to_uniform(SEED, c, model.latent_dim), 50, rng_key=(SEED, c))
        seq = []
        for it in range(8):
            ost = sample_kernel(ost)
            seq.append(ost.adapt_state.step_size)
        # the first transitions must agree for every chain; later ones may part
        # once FP32-vs-FP64 rounding is amplified by the (chaotic) dynamics
        np.testing.assert_allclose(np.array(seq[:3]), gpu_steps[:3, c], rtol=1e-4)
        if np.allclose(np.array(seq), gpu_steps[:, c], rtol=1e-4):
            agree += 1
    assert agree >= C // 2, agree
    k.close()


@pytest.mark.gpu
def test_hmc_fixed_steps_parity():
    model, pot = _hier()
    C = 64
    k = HMC(model, num_chains=C, step_size=0.1, num_steps=7, trajectory_length=None, adapt_step_size=False,
            adapt_mass_matrix=False)
    st = k.init(SEED, 0)
    z0 = st.z.cpu().numpy()
    new = k.sample(st)
    zg = new.z.cpu().numpy()
    ap = new.accept_prob.cpu().numpy()
    for c in range(C):
        ref = _oracle_transition(pot, z0[c], 0.1, np.ones(model.latent_dim), c, 0, algo="HMC", traj=None, nsteps=7)
        assert new.num_steps.cpu().numpy()[c] == 7
        assert abs(ref.accept_prob - ap[c]) < 1e-4
        np.testing.assert_allclose(zg[c], ref.z, rtol=1e-5, atol=1e-5)
    k.close()


@pytest.mark.gpu
def test_divergence_large_step():
    """test/infer/test_hmc_util.py:406-442 invariant: huge steps diverge in one leaf."""
    model, _ = _hier()
    k = NUTS(model, num_chains=16, step_size=100.0, adapt_step_size=False)
    st = k.sample(k.init(SEED, 0))
    assert bool(st.diverging.all())
    assert int(st.num_steps.max()) == 1
    k.close()


@pytest.mark.gpu
def test_uneven_batched_models_match_single_model_runs():
    """One launch over models of different J gives each model the result of running it alone."""
    ds = datasets.uneven_hierarchical(seed=0, num_models=6, jmin=3, jmax=20)
    batched = models.HierarchicalNormal(datasets=ds)
    kb = NUTS(batched, num_chains=12)
    sb = kb.init(SEED, 30)
    outb = kb.run_device(sb, 40, collect_start=30, collect=("z",))["z"].cpu().numpy()
    kb.close()
    # model 2 alone with the same chain ids (4, 5) -> same stream addresses
    m2 = models.HierarchicalNormal(*ds[2])
    k2 = NUTS(m2, num_chains=6)
    s2 = k2.init(SEED, 30)
    out2 = k2.run_device(s2, 40, collect_start=30, collect=("z",))["z"].cpu().numpy()
    k2.close()
    D2 = m2.latent_dim
    np.testing.assert_array_equal(outb[4:6, :, :D2], out2[4:6])
    assert np.all(outb[4:6, :, D2:] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("family", ["hier", "logreg"])
def test_tick_graph_replay_matches_direct_launches(family, monkeypatch):
    """Batches of ticks replayed from a captured CUDA graph give the draws of launching every
    kernel directly (GBN_CUDA_GRAPHS=0), bit for bit."""
    if family == "hier":
        model, _ = _hier()
        C, kw = 16, dict(engine="ticks")
    else:
        X, yv, _ = datasets.covtype_like(seed=5, n=4000, n_cont=3, n_bin=4)
        model = models.LogisticRegression(X, yv)
        C, kw = 64, dict(engine="fused", precision="fp32")
    res = []
    for graphs in ("1", "0"):
        monkeypatch.setenv("GBN_CUDA_GRAPHS", graphs)
        k = NUTS(model, num_chains=C, **kw)
        st = k.init(SEED, 40)
        out = k.run_device(st, 80, collect_start=0, collect=("z", "num_steps"))
        res.append((out["z"].cpu().numpy(), out["num_steps"].cpu().numpy()))
        k.close()
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])


@pytest.mark.gpu
def test_fused_tensor_core_tick_matches_separate_split_and_finish(monkeypatch):
    """The tick engine folds the tensor-core logistic potential's coefficient split and row-group
    finish into its state-machine kernel (two launches per tick instead of four); with
    GBN_FUSE_TICK=0 they run as their own kernels.  Both forms share the arithmetic, so the draws
    and tree sizes agree bit for bit, through warmup and sampling, and through the device-side
    loop of gbn_sample_async."""
    X, yv, _ = datasets.covtype_like(seed=6, n=20_000)
    model = models.LogisticRegression(X, yv)
    res = []
    for fuse in ("1", "0"):
        monkeypatch.setenv("GBN_FUSE_TICK", fuse)
        k = NUTS(model, num_chains=256, precision="bf16x3")
        st = k.init(SEED, 60)
        out = k.run_device(st, 100, collect_start=0, collect=("z", "num_steps"))
        for _ in range(3):
            st = k.sample_async(st)
        k.check_async()
        res.append((out["z"].cpu().numpy(), out["num_steps"].cpu().numpy(), st.z.cpu().numpy(),
                     st.potential_energy.cpu().numpy()))
        k.close()
    for a, b in zip(res[0], res[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("noncentered", [True, False])
def test_fused_horseshoe_tick_matches_separate_split_and_finish(monkeypatch, noncentered):
    """The same fusion for the tensor-core horseshoe potential, where the state machine runs a CTA
    per chain (latent dimension > 1024; below that the warp-per-chain kernel runs and the split and
    finish stay separate kernels): the state-machine kernel writes the coefficients' bf16 terms of
    each queried position and finishes the previous potential (hs_finish.cuh), leaving the two
    GEMMs as the tick's other launches.  With GBN_FUSE_TICK=0 the split and finish run as their
    own kernels.  Bit-identical draws."""
    X, yv, _ = datasets.horseshoe_data(seed=3, n=600, p=520, nonzero=5)
    model = models.HorseshoeRegression(X, yv, noncentered=noncentered)
    assert model.latent_dim > 1024
    res = []
    for fuse in ("1", "0"):
        monkeypatch.setenv("GBN_FUSE_TICK", fuse)
        k = NUTS(model, num_chains=128, precision="bf16x3")
        st = k.init(SEED, 40)
        out = k.run_device(st, 60, collect_start=0, collect=("z", "num_steps"))
        res.append((out["z"].cpu().numpy(), out["num_steps"].cpu().numpy(), st.z.cpu().numpy(),
                    st.potential_energy.cpu().numpy()))
        k.close()
    for a, b in zip(res[0], res[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.gpu
def test_chains_split_over_kernels_keep_their_draws():
    """first_chain: every draw is addressed by (seed, global chain id, ...), so 128 chains run as two
    kernels of 64 (global ids 0-63 and 64-127, one seed) give the draws of one kernel of 128, chain
    for chain -- how bench.py shards replicas over GPUs."""
    y, s = datasets.eight_schools(0)
    model = models.HierarchicalNormal(y, s)
    whole = NUTS(model, num_chains=128)
    st = whole.init(SEED, 100)
    ref = whole.run_device(st, 150, collect_start=100, collect=("z", "num_steps"))
    ref = (ref["z"].cpu().numpy(), ref["num_steps"].cpu().numpy())
    whole.close()
    parts = []
    for r in range(2):
        k = NUTS(model, num_chains=64, first_chain=64 * r)
        st = k.init(SEED, 100)
        out = k.run_device(st, 150, collect_start=100, collect=("z", "num_steps"))
        parts.append((out["z"].cpu().numpy(), out["num_steps"].cpu().numpy()))
        k.close()
    np.testing.assert_array_equal(np.concatenate([p[0] for p in parts]), ref[0])
    np.testing.assert_array_equal(np.concatenate([p[1] for p in parts]), ref[1])
