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
one of 1,024 may part), median relative position error of the agreeing transitions < 1e-5,
and accept probabilities within 5e-3 at the 99th percentile (the mean of min(1, e^-dE) over
the leaves; the FP32 energy of a 4,098-dimensional potential carries ~1e-3 of absolute
rounding, measured 2.5e-3 at most for stochastic volatility, 3e-5 for the logistic model).

Horseshoe at P = 1000: after warmup the trees run to ~1,000 leapfrog steps, long enough for
float32 rounding alone to move a U-turn or divergence decision: the FP32 build of the same C
restatement, replayed from the same states, parts from FP64 on ~2-4 % of the transitions.
The bar there is relative to that: the GPU must agree with FP64 at least as often as the
float32 restatement does, less 1 % of the transitions, and on >= 97 % in any case; its
median position error and 99th-percentile accept-probability error may be at most 3 times
the float32 restatement's (and are held to the FP32 bars above when those are larger).

bf16x3 logistic: the gradient's E = tanh(X'b/2) enters the tensor cores rounded to bfloat16
(absolute error <= 2^-9 per row), and where the kernel takes the coefficients as two bf16 terms
with a first-order energy term, the gradient is the one at that two-term value (2^-16 relative);
the energies (and so the acceptance and the multinomial choice) stay exact to FP32.  The leapfrog
with any deterministic gradient field is still volume-preserving and reversible, so the target is
unchanged; only the trajectory moves.  Measured on GB300: tree sizes identical on 1,024 of 1,024
transitions, median position error 6.3e-4, accept probabilities within 6e-3 (3.7e-3 and 2e-2 when E
was sigmoid(X'b) in bfloat16).  Bar: tree sizes >= 99 %, median position error < 1e-2, accept
probabilities within 5e-2.
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


def _check(res, name, min_frac=0.999, zerr_median=1e-5, ap_tol=5e-3):
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
        _check(res, "logistic bf16x3", min_frac=0.99, zerr_median=1e-2, ap_tol=5e-2)


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
    res = replay_parity(k, st, cmodel_of(model), SEED, TRANSITIONS, fp32_oracle=True)
    k.close()
    total, same32 = res["total"], res["same32"]
    print("horseshoe_nc P=1000: the FP32 restatement agrees with FP64 on %d of %d transitions (%.4f)"
          % (same32, total, same32 / total))
    z32, a32 = np.median(res["zerr32"]), np.percentile(res["aperr32"], 99)
    print("FP32 restatement vs FP64: median position error %.2e, 99th pct accept-prob error %.2e" % (z32, a32))
    bar = max(0.97, min(0.999, same32 / total - 0.01))
    _check(res, "horseshoe_nc P=1000 %s" % precision, min_frac=bar, zerr_median=max(1e-5, 3 * z32),
           ap_tol=max(5e-3, 3 * a32))


@pytest.mark.gpu
def test_uneven_hierarchical_batch_transitions():
    ds = datasets.uneven_hierarchical(seed=7, num_models=64, jmin=4, jmax=256)
    model = models.HierarchicalNormal(datasets=ds)
    k, st = _warm(model, 300)
    res = replay_parity(k, st, cmodel_of(model, chains_per_model=CHAINS // 64), SEED, TRANSITIONS)
    k.close()
    _check(res, "uneven hierarchical (64 models, J 4..256) persistent")
