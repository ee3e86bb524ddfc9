"""The allocation-free logistic potential (gbn_logreg_potential_noalloc).

It exists for callers that cannot call cudaMalloc when a potential is needed --
a JAX/XLA FFI handler, code inside a CUDA stream capture, hosts with their own
memory pool -- and keeps its scratch in a static device array instead.  Here it
is called through the C ABI with device buffers and must agree with the
allocating entry point (gbn_potential_and_grad on a LOGREG handle), within the
potential tolerances used by the other GPU tests, on two calls in a row.  This
file is collected last so that a failure here never hides the other tests.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice():
    from numpyro_gb300 import NUTS, _lib, datasets, models

    lib = _lib.load()
    X, y, beta = datasets.covtype_like(seed=4, n=5000, n_cont=6, n_bin=4)
    n, p = X.shape
    C = 200
    model = models.LogisticRegression(X, y)
    ref_kernel = NUTS(model, num_chains=C, precision="fp32")
    dx = torch.as_tensor(X, device="cuda").contiguous()
    dy = torch.as_tensor(y, device="cuda").contiguous()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(0)
    for call in range(2):
        z = torch.as_tensor((beta[None, :] + 0.3 * rng.standard_normal((C, p))).astype(np.float32), device="cuda")
        pe = torch.full((C,), float("nan"), dtype=torch.float64, device="cuda")
        g = torch.full((C, p), float("nan"), dtype=torch.float32, device="cuda")
        status = lib.gbn_logreg_potential_noalloc(stream, _ptr(dx), _ptr(dy), n, p, 1.0, _ptr(z), C, _ptr(pe),
                                                  _ptr(g))
        assert status == 0, lib.gbn_noalloc_last_error()
        pe_ref, g_ref = ref_kernel.potential_and_grad(z)
        torch.cuda.synchronize()
        pe, g, pe_ref, g_ref = (t.cpu().numpy() for t in (pe, g, pe_ref, g_ref))
        np.testing.assert_allclose(pe, pe_ref, rtol=2e-6, err_msg="call %d" % call)
        scale = np.max(np.abs(g_ref), axis=1, keepdims=True)
        assert np.max(np.abs(g - g_ref) / np.maximum(scale, 1.0)) < 1e-3, "call %d" % call
    ref_kernel.close()


@pytest.mark.gpu
def test_noalloc_rejects_too_many_points():
    from numpyro_gb300 import _lib

    lib = _lib.load()
    d = torch.zeros(8, device="cuda")
    too_many = _lib.NOALLOC_MAX_POINTS + 1
    status = lib.gbn_logreg_potential_noalloc(None, _ptr(d), _ptr(d), 2, 2, 1.0, _ptr(d), too_many, _ptr(d),
                                              _ptr(d))
    assert status == 1
    assert b"GBN_NOALLOC_MAX_POINTS" in lib.gbn_noalloc_last_error()
