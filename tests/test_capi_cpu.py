"""CPU-only checks of the C ABI and host logic (no kernel is launched here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbnuts.h")


def _declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gbn_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = _declared_symbols()
    for s in ["gbn_create", "gbn_destroy", "gbn_init", "gbn_sample", "gbn_run", "gbn_potential_and_grad",
              "gbn_potential_vjp", "gbn_last_error", "gbn_abi_version", "gbn_get_stats", "gbn_latent_dim"]:
        assert s in syms


def test_library_loads_and_exports_every_declared_symbol():
    from numpyro_gb300 import _lib, build

    build.build()
    lib = ctypes.CDLL(_lib.LIB_PATH)
    for s in _declared_symbols():
        assert hasattr(lib, s), s
    assert lib.gbn_abi_version() == 2


def test_struct_layouts_match_header():
    """ctypes mirrors of the header structs have the C sizes (checked by compiling a probe)."""
    import subprocess
    import tempfile

    from numpyro_gb300 import _lib

    src = r"""
#include <stdio.h>
#include "gbnuts.h"
int main(void){printf("%zu %zu %zu %zu %zu\n", sizeof(gbn_model_desc), sizeof(gbn_config),
  sizeof(gbn_state), sizeof(gbn_collect), sizeof(gbn_stats));return 0;}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        sizes = [int(v) for v in subprocess.check_output([exe]).split()]
    assert sizes == [ctypes.sizeof(_lib.ModelDesc), ctypes.sizeof(_lib.Config), ctypes.sizeof(_lib.State),
                     ctypes.sizeof(_lib.Collect), ctypes.sizeof(_lib.Stats)]


def test_kernel_constructor_contract():
    from numpyro_gb300 import NUTS, HMC, models

    m = models.HierarchicalNormal(np.zeros(3), np.ones(3))
    k = NUTS(m, max_tree_depth=(8, 10), target_accept_prob=0.9)
    assert k.sample_field == "z" and k.default_fields == ("z", "diverging")
    with pytest.raises(ValueError):
        NUTS()
    with pytest.raises(NotImplementedError):
        NUTS(potential_fn=lambda z: z)
    assert NUTS(m, dense_mass=True)._dense_mass
    # block-structured dense mass (numpyro's list of site tuples): per-coordinate block ids
    k = NUTS(m, dense_mass=[("theta_base", "mu")])
    assert k._dense_mass
    sl = m.site_slices()
    expect = np.full(m.latent_dim, -1, np.int32)
    expect[sl["mu"][0]:sl["mu"][1]] = 0
    expect[sl["theta_base"][0]:sl["theta_base"][1]] = 0
    np.testing.assert_array_equal(k._mass_blocks, expect)
    k = NUTS(m, dense_mass=[("mu",), ("tau", "theta_base")])
    assert list(k._mass_blocks[:2]) == [0, 1] and set(k._mass_blocks[2:]) == {1}
    assert not NUTS(m, dense_mass=[])._dense_mass
    for bad in ([("mu", "nope")], [("mu",), ("mu", "tau")], ["mu"], "mu"):
        with pytest.raises(ValueError):
            NUTS(m, dense_mass=bad)
    with pytest.raises(ValueError):
        HMC(m, num_steps=None, trajectory_length=None)


def test_model_layout_sorted_sites():
    from numpyro_gb300 import models

    m = models.HorseshoeRegression(np.zeros((5, 3)), np.zeros(5))
    assert [s.name for s in m.sites] == sorted(s.name for s in m.sites)
    assert m.latent_dim == 8
    out = m.postprocess(np.zeros(8))
    assert out["sigma"].item() == 1.0 and out["beta"].shape == (3,)
    hn = models.HorseshoeRegression(np.zeros((5, 3)), np.zeros(5), noncentered=True)
    assert [s.name for s in hn.sites] == ["lambdas", "sigma", "tau", "unscaled_betas"]
    zz = np.concatenate([np.zeros(3), [0.0, np.log(2.0)], [1.0, 2.0, 3.0]])
    np.testing.assert_allclose(hn.postprocess(zz)["beta"], [2.0, 4.0, 6.0])
    sv = models.StochasticVolatility(np.zeros(10))
    assert [s.name for s in sv.sites] == ["h", "nu", "s"] and sv.latent_dim == 12
    nc = models.StochasticVolatility(np.zeros(10), noncentered=True)
    assert [s.name for s in nc.sites] == ["h_base", "nu", "s"] and nc.latent_dim == 12
    z = np.concatenate([np.ones(10), [0.0, np.log(0.5)]])
    np.testing.assert_allclose(nc.postprocess(z)["h"], 0.5 * np.arange(1, 11))


def test_adaptation_schedule_host_matches_oracle():
    """The C++ schedule is checked on device; the Python oracle table pins the reference."""
    from oracle import nuts_ref as R

    assert R.build_adaptation_schedule(500)[-1] == R.AdaptWindow(450, 499)


# ---- diagnostics known answers: test/test_diagnostics.py:61-108
def test_autocorrelation_known_answer():
    from numpyro_gb300.diagnostics import autocorrelation, autocovariance

    x = np.arange(10.0)
    np.testing.assert_allclose(autocorrelation(x, bias=False),
                               [1, 0.78, 0.52, 0.21, -0.13, -0.52, -0.94, -1.4, -1.91, -2.45], atol=0.01)
    np.testing.assert_allclose(autocovariance(x, bias=False),
                               [8.25, 6.42, 4.25, 1.75, -1.08, -4.25, -7.75, -11.58, -15.75, -20.25], atol=0.01)


def test_gelman_rubin_known_answer():
    from numpyro_gb300.diagnostics import gelman_rubin, split_gelman_rubin

    x = np.empty((2, 10))
    x[0] = np.arange(10.0)
    x[1] = np.arange(10.0) + 1
    np.testing.assert_allclose(gelman_rubin(x), 0.98, atol=0.01)
    y = np.random.default_rng(0).normal(size=(2, 10))
    np.testing.assert_allclose(gelman_rubin(y.reshape(2, 2, 5).reshape(4, 5)), split_gelman_rubin(y))


def test_effective_sample_size_known_answer():
    from numpyro_gb300.diagnostics import effective_sample_size

    x = np.arange(1000.0).reshape(100, 10)
    np.testing.assert_allclose(effective_sample_size(x, bias=False), 52.64, atol=0.01)


def test_fft_next_fast_len():
    from scipy.fftpack import next_fast_len

    from numpyro_gb300.diagnostics import _fft_next_fast_len

    for t in [433, 124, 25, 300, 1, 3, 7]:
        assert _fft_next_fast_len(t) == next_fast_len(t)


def test_bulk_ess_iid():
    from numpyro_gb300.diagnostics import bulk_effective_sample_size

    x = np.random.default_rng(1).normal(size=(4, 1000))
    ess = bulk_effective_sample_size(x)
    assert 3000 < ess < 5000


def test_bf16_rounding_exact():
    from numpyro_gb300.datasets import _round_bf16

    a = np.random.default_rng(0).normal(size=1000).astype(np.float32)
    r = _round_bf16(a)
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)
    assert np.max(np.abs(r - a) / np.abs(a)) <= 2.0 ** -8


def test_transfer_states_to_host_converts_tensors():
    """MCMC.transfer_states_to_host (numpyro/infer/mcmc.py:799-804) leaves host arrays only."""
    import torch

    from numpyro_gb300.mcmc import MCMC

    class _Kernel:
        sample_field = "z"
        default_fields = ("z", "diverging")

    m = MCMC(_Kernel(), num_warmup=1, num_samples=2, num_chains=2)
    m._states = {"z": {"mu": torch.zeros(2, 2), "tau": np.ones((2, 2))}, "diverging": torch.zeros(2, 2)}
    m.transfer_states_to_host()
    assert isinstance(m._states["z"]["mu"], np.ndarray) and isinstance(m._states["diverging"], np.ndarray)
    assert m.get_samples()["mu"].shape == (4,)


def test_diagnostic_entry_points_reject_null_arguments():
    """gbn_logreg_terms and gbn_measure_sfu check their arguments before touching the GPU."""
    from numpyro_gb300 import _lib

    lib = _lib.load()
    three, blocks, limit = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_float()
    invalid = 1  # GBN_ERR_INVALID_ARG
    assert lib.gbn_logreg_terms(None, ctypes.byref(three), ctypes.byref(blocks), ctypes.byref(limit)) == invalid
    assert b"null argument" in lib.gbn_last_error(None)
    assert lib.gbn_measure_sfu(None, 7, ctypes.byref(ctypes.c_double())) == invalid
