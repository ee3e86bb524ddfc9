"""NUTS transition parity at the benchmark shapes: CUDA engines vs the FP64 C oracle.

Every engine path that runs a benchmark configuration is checked here:
  * the covtype-shaped logistic model (55 coefficients, 50,000 rows) on FP32 CUDA cores and
    on the bf16x3 tensor cores;
  * stochastic volatility at T = 4096 (a CTA per chain) on the tick and persistent engines;
  * the non-centred horseshoe at N = 2000, P = 1000 on FP32 CUDA cores and bf16x3 tensor cores;
  * a batch of 64 uneven hierarchical models (J from 4 to 256) on the persistent engine.
256 chains are warmed up on the GPU (Stan windows, dual averaging), then 4 transitions of
every chain are replayed by the FP64 C oracle (oracle/nuts_ref.c; pinned to the Python
restatement, which is pinned to numpyro's own known answers) from the GPU's own starting
state with the same Philox bits: 1,024 transitions per case.

Bar (build_tree, numpyro/infer/hmc_util.py:1088-1180, in numpyro's float32 dtype against
FP64): tree sizes and divergence flags identical on >= 99.9 % of the transitions (at most
one of 1,024 may part), accept probabilities within 1e-3, median relative position error
of the agreeing transitions < 1e-5.

bf16x3 logistic: the gradient's residual E = sigmoid(X'b) enters the tensor cores rounded
to bfloat16 (relative error <= 2^-9 per row); the energies (and so the acceptance and the
multinomial choice) stay exact to FP32.  Per leapfrog step the gradient then differs from
FP32 by ~1e-3 of its scale, so trajectories part from the FP64 ones by ~1e-3 relative
after tens of steps; tree sizes still agree on >= 99 % and the median position error is
< 2e-3 (the measured agreement is printed).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import NUTS, datasets, models  # noqa: E402

from gpu_helpers import cmodel_of, replay_parity  # noqa: E402

SEED = 4321
CHAINS = 256
TRANSITIONS = 4


def _warm(model, num_warmup, **kw):
    k = NUTS(model, num_chains=CHAINS, **kw)
    st = k.init(SEED, num_warmup)
    k.run_device(st, num_warmup, collect_start=num_warmup)
    torch.cuda.synchronize()
    return k, st


def _check(res, name, min_frac=0.999, zerr_median=1e-5, ap_tol=1e-3):
    frac, zerr, aperr = res["frac"], res["zerr"], res["aperr"]
    print("%s: tree sizes identical on %d of %d transitions (%.4f); median position error %.2e, "
          "95th pct %.2e; max accept-prob error %.2e"
          % (name, res["same"], res["total"], frac, np.median(zerr), np.percentile(zerr, 95), aperr.max()))
    assert frac >= min_frac, (name, frac)
    assert np.median(zerr) < zerr_median, (name, np.median(zerr))
    assert np.percentile(aperr, 99) <= ap_tol, (name, np.percentile(aperr, 99))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_logistic_covtype_shape_transitions(precision):
    X, y, _ = datasets.covtype_like(seed=3, n=50_000)
    model = models.LogisticRegression(X, y)
    k, st = _warm(model, 200, precision=precision)
    res = replay_parity(k, st, cmodel_of(model), SEED, TRANSITIONS)
    k.close()
    if precision == "fp32":
        _check(res, "logistic fp32")
    else:
        _check(res, "logistic bf16x3", min_frac=0.99, zerr_median=2e-3, ap_tol=5e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ["ticks", "fused"])
def test_stochastic_volatility_T4096_transitions(engine):
    r, _ = datasets.sv_returns(seed=0, T=4096)
    model = models.StochasticVolatility(r)
    k, st = _warm(model, 300, engine=engine)
    res = replay_parity(k, st, cmodel_of(model), SEED, TRANSITIONS)
    k.close()
    _check(res, "sv T=4096 %s" % engine)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_horseshoe_P1000_transitions(precision):
    X, y, _ = datasets.horseshoe_data(seed=0, n=2000, p=1000)
    model = models.HorseshoeRegression(X, y, noncentered=True)
    k, st = _warm(model, 150, precision=precision)
    res = replay_parity(k, st, cmodel_of(model), SEED, TRANSITIONS)
    k.close()
    _check(res, "horseshoe_nc P=1000 %s" % precision)


@pytest.mark.gpu
def test_uneven_hierarchical_batch_transitions():
    ds = datasets.uneven_hierarchical(seed=7, num_models=64, jmin=4, jmax=256)
    model = models.HierarchicalNormal(datasets=ds)
    k, st = _warm(model, 300)
    res = replay_parity(k, st, cmodel_of(model, chains_per_model=CHAINS // 64), SEED, TRANSITIONS)
    k.close()
    _check(res, "uneven hierarchical (64 models, J 4..256) persistent")
