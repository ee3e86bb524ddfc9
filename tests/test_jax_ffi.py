"""The jax side of the boundary (numpyro_gb300/jax_ffi.py, csrc/xla_ffi.cc).

numpyro runs ``sample`` under ``jit`` (numpyro/infer/mcmc.py:188-190) and differentiates
``potential_fn`` (numpyro/infer/hmc_util.py:242-252); jax.ffi custom calls stand in for both.
jax is not installed in this container nor on the GPU machine, so the tests that call through XLA
skip with that reason; the guard itself, the build's recorded reason and the handle registry
the handlers use are tested everywhere (the registry on the GPU).
"""
import numpy as np
import pytest


def test_jax_path_reports_why_it_cannot_run():
    from numpyro_gb300 import jax_ffi

    why = jax_ffi.unavailable()
    try:
        import jax  # noqa: F401
    except ImportError:
        assert why and "jax" in why
        with pytest.raises(RuntimeError, match="jax"):
            jax_ffi.register()
    assert jax_ffi.STATE_FIELDS[0] == "i" and len(jax_ffi.STATE_FIELDS) == 19


def test_build_records_why_the_xla_handlers_were_not_built():
    from numpyro_gb300 import build

    inc, why = build.xla_ffi_include()
    assert (inc is None) == (why is not None)
    if inc is None:
        assert build.build_xla_ffi() is None and build.XLA_FFI_STATUS == why


def test_handler_source_binds_the_c_abi():
    import os

    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "numpyro_gb300",
                            "csrc", "xla_ffi.cc")).read()
    for sym in ("gbn_xla_potential_and_grad", "gbn_xla_potential_vjp", "gbn_xla_sample", "gbn_handle_from_id",
                "gbn_sample_async", "gbn_potential_vjp"):
        assert sym in src, sym


@pytest.mark.gpu
def test_handle_registry_round_trip():
    from numpyro_gb300 import NUTS, _lib, datasets, models

    lib = _lib.load()
    y, s = datasets.eight_schools(0)
    k1 = NUTS(models.HierarchicalNormal(y, s), num_chains=4)
    k2 = NUTS(models.HierarchicalNormal(y, s), num_chains=4)
    k1.init(1, 0)
    k2.init(1, 0)
    i1, i2 = lib.gbn_handle_id(k1._handle), lib.gbn_handle_id(k2._handle)
    assert i1 > 0 and i2 > 0 and i1 != i2
    hv = k1._handle.value if hasattr(k1._handle, "value") else k1._handle
    assert lib.gbn_handle_from_id(i1) == hv
    k1.close()
    assert not lib.gbn_handle_from_id(i1)
    assert lib.gbn_handle_from_id(i2)
    k2.close()
    assert lib.gbn_handle_id(None) == 0


@pytest.mark.gpu
def test_potential_through_xla_matches_the_c_abi():
    jax = pytest.importorskip("jax", reason="jax is not installed on this machine: the XLA FFI path cannot run")
    from numpyro_gb300 import NUTS, datasets, jax_ffi, models

    if jax_ffi.unavailable():
        pytest.skip(jax_ffi.unavailable())
    jax.config.update("jax_enable_x64", True)
    X, yv, _ = datasets.covtype_like(seed=1, n=3000, n_cont=4, n_bin=6)
    k = NUTS(models.LogisticRegression(X, yv), num_chains=8)
    k.init(0, 0)
    z = np.random.default_rng(0).standard_normal((8, X.shape[1])).astype(np.float32) * 0.3
    pe, g = jax_ffi.potential_and_grad(k, z)
    import torch

    pe_ref, g_ref = k.potential_and_grad(torch.as_tensor(z, device="cuda"))
    np.testing.assert_allclose(np.asarray(pe), pe_ref.cpu().numpy(), rtol=1e-12)
    np.testing.assert_allclose(np.asarray(g), g_ref.cpu().numpy(), rtol=1e-6)
    U = jax_ffi.potential_fn(k)
    gv = jax.grad(lambda zz: U(zz).sum())(z)
    np.testing.assert_allclose(np.asarray(gv), g_ref.cpu().numpy(), rtol=1e-6)
    k.close()
