"""Warmup adaptation on the GPU against the FP64 oracle, through the window ends.

numpyro's warmup_adapter (numpyro/infer/hmc_util.py:518-707) runs dual averaging every
warmup iteration, a diagonal Welford estimate in the middle (slow) windows, and at the end
of each slow window finalises the mass matrix (welford_covariance.final_fn, :199-239, with
the Stan regularisation), resets the Welford state and re-initialises dual averaging
(:596-635, :698-704).  At the last warmup iteration the step size switches to
exp(x_avg) (:665-669).  find_reasonable_step_size (:314-384) runs at init and, when asked,
at every slow-window end.

Long warmups are chaotic (FP32 against FP64 rounding grows along the dynamics), so each
window end is checked by replay: the GPU warmup runs up to two iterations before the end,
its complete adaptation state (position, step size, mass matrix rows, dual-averaging
state, Welford mean/m2/count, window index) is handed to the oracle, and both then run the
same transitions across the window end with the same Philox bits.  Windows for 200 warmup
iterations end at 74, 99, 149 and 199, so the slow windows end at 99 and 149.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from numpyro_gb300 import NUTS, datasets, models  # noqa: E402
from oracle import nuts_ref as R  # noqa: E402
from oracle import potentials_ref as PR  # noqa: E402

SEED = 2468
NUM_WARMUP = 200


def _hier():
    y, s = datasets.eight_schools(0)
    return models.HierarchicalNormal(y, s), PR.make_potential("hier_nc", y.astype(np.float64), s.astype(np.float64))


def _snapshot(st):
    a = st.adapt_state
    return {
        "i": st.i.cpu().numpy().copy(), "z": st.z.cpu().numpy().astype(np.float64),
        "step": a.step_size.cpu().numpy().copy(), "inv": a.inverse_mass_matrix.cpu().numpy().astype(np.float64),
        "msq": a.mass_matrix_sqrt.cpu().numpy().astype(np.float64),
        "msqi": a.mass_matrix_sqrt_inv.cpu().numpy().astype(np.float64),
        "ss": a.ss_state.cpu().numpy().copy(), "mean": a.mm_state[0].cpu().numpy().copy(),
        "m2": a.mm_state[1].cpu().numpy().copy(), "n": a.mm_state[2].cpu().numpy().copy(),
        "widx": a.window_idx.cpu().numpy().copy(), "key": st.rng_key.cpu().numpy().astype(np.int64),
    }


def _oracle_from_snapshot(pot, snap, c, **kw):
    """An oracle chain (init_kernel closures for NUM_WARMUP) carrying the GPU's state of chain c."""
    init_kernel, sample_kernel = R.hmc(pot)
    z = snap["z"][c]
    st = init_kernel(z, NUM_WARMUP, rng_key=(SEED, c), **kw)
    ss = snap["ss"][c]
    adapt = R.HMCAdaptState(float(snap["step"][c]), snap["inv"][c], snap["msq"][c], snap["msqi"][c],
                            (float(ss[0]), float(ss[1]), float(ss[2]), int(round(ss[3])), float(ss[4])),
                            (snap["mean"][c].copy(), snap["m2"][c].copy(), int(snap["n"][c])),
                            int(snap["widx"][c]), None)
    pe, g = pot(z)
    st = st._replace(i=int(snap["i"][c]), z=z, z_grad=g, potential_energy=pe, adapt_state=adapt,
                     rng_key=R.RngKey(SEED, c, int(snap["key"][c, 1])))
    return st, sample_kernel


def _run_across(k, st, pot, until, steps, C, **kw):
    """GPU warmup to iteration `until`, then `steps` GPU and oracle transitions side by side."""
    k.run_device(st, until - int(st.i[0]), collect_start=until)
    snap = _snapshot(st)
    assert np.all(snap["i"] == until)
    gpu = []
    cur = st
    for _ in range(steps):
        cur = k.sample(cur)
        gpu.append(_snapshot(cur) | {"ns": cur.num_steps.cpu().numpy().copy()})
    agree = 0
    for c in range(C):
        ost, sample_kernel = _oracle_from_snapshot(pot, snap, c, **kw)
        ok = True
        for s in range(steps):
            ost = sample_kernel(ost)
            g = gpu[s]
            a = ost.adapt_state
            if ost.num_steps != g["ns"][c]:
                ok = False
                break
            assert a.window_idx == g["widx"][c], (c, s, a.window_idx, g["widx"][c])
            # dual averaging turns an accept-probability difference da into a relative step-size
            # difference of sqrt(t) / (gamma (t + t0)) da, 1.8 da at t = 1 just after a window end;
            # FP32 accept probabilities agree with FP64 to ~1e-3, hence 2e-3
            np.testing.assert_allclose(g["step"][c], a.step_size, rtol=2e-3, err_msg="chain %d step %d" % (c, s))
            np.testing.assert_allclose(g["inv"][c], a.inverse_mass_matrix, rtol=1e-4, atol=1e-7,
                                       err_msg="chain %d step %d" % (c, s))
            np.testing.assert_allclose(g["msq"][c], a.mass_matrix_sqrt, rtol=1e-4,
                                       err_msg="chain %d step %d" % (c, s))
            assert g["n"][c] == a.mm_state[2], (c, s)
            # the prox centre log(10 step) carries the step size's relative error as an absolute one
            np.testing.assert_allclose(g["ss"][c][4], a.ss_state[4], rtol=0, atol=2e-3)
        agree += ok
    return agree, cur


@pytest.mark.gpu
@pytest.mark.parametrize("heuristic", [False, True])
def test_diagonal_warmup_across_slow_window_ends(heuristic):
    model, pot = _hier()
    C = 32
    kw = dict(find_heuristic_step_size=heuristic)
    k = NUTS(model, num_chains=C, **kw)
    st = k.init(SEED, NUM_WARMUP)
    # slow-window end 99: iterations 97, 98, 99 (window end: mass matrix, reset), 100
    agree, st = _run_across(k, st, pot, 97, 4, C, **kw)
    print("window end 99: %d of %d chains identical through the window end" % (agree, C))
    assert agree >= C - 1, agree
    # slow-window end 149
    agree, st = _run_across(k, st, pot, 147, 4, C, **kw)
    print("window end 149: %d of %d chains identical through the window end" % (agree, C))
    assert agree >= C - 1, agree
    # the last warmup iteration (199) switches the step size to exp(x_avg); 200 samples
    agree, st = _run_across(k, st, pot, 197, 4, C, **kw)
    print("end of warmup: %d of %d chains identical" % (agree, C))
    assert agree >= C - 1, agree
    a = st.adapt_state
    assert np.all(a.window_idx.cpu().numpy() == 4)
    # after warmup the step size is exp(x_avg) of the final dual-averaging state
    ss = a.ss_state.cpu().numpy()
    np.testing.assert_allclose(a.step_size.cpu().numpy(), np.exp(ss[:, 1]).astype(np.float32), rtol=1e-6)
    k.close()


@pytest.mark.gpu
def test_find_heuristic_step_size_at_init_matches_oracle():
    """hmc.py:320-323 -> find_reasonable_step_size at init: the step size doubles or halves from
    1.0 until the acceptance crosses 0.8, so the result is a power of two and must be exact."""
    model, pot = _hier()
    C = 64
    k = NUTS(model, num_chains=C, find_heuristic_step_size=True)
    st = k.init(SEED, 50)
    gpu = st.adapt_state.step_size.cpu().numpy()
    z0 = st.z.cpu().numpy()
    same = 0
    for c in range(C):
        init_kernel, _ = R.hmc(pot)
        o = init_kernel(z0[c].astype(np.float64), 50, find_heuristic_step_size=True, rng_key=(SEED, c))
        same += np.float32(o.adapt_state.step_size) == gpu[c]
        assert math.log2(gpu[c]) == round(math.log2(gpu[c]))
    print("heuristic step size identical for %d of %d chains" % (same, C))
    assert same >= C - 1, same
    # dual averaging starts from log(10 * step_size)
    ss = st.adapt_state.ss_state.cpu().numpy()
    np.testing.assert_allclose(ss[:, 4], np.log(10.0 * gpu.astype(np.float64)), rtol=1e-12)
    k.close()
