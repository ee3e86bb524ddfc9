"""The allocation-free logistic potential (gbn_logreg_potential_noalloc).

It exists for callers that cannot call cudaMalloc when a potential is needed --
a JAX/XLA FFI handler, whose device memory XLA owns, or a host that routes all
device memory through its own pool -- and keeps its scratch in a static device
array instead.  Here it is called through the C ABI with device buffers, on two
calls in a row of different sizes (the second with fewer chains and fewer rows,
so fewer row groups than the first: stale scratch from the first call would
show), and must agree with the FP64 oracle and with the allocating entry point
(gbn_potential_and_grad on a LOGREG handle) within the tolerances of the other
potential tests.  This file is collected last so that a failure here never
hides the other tests.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.gpu
def test_noalloc_matches_oracle_and_allocating_entry_point_twice():
    from numpyro_gb300 import NUTS, _lib, datasets, models
    from oracle import potentials_ref as PR

    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(0)
    # (rows, chains): 5000 rows = 79 row tiles (16 row groups), then 700 rows = 11 row groups
    for call, (n_rows, C, seed) in enumerate([(5000, 200, 4), (700, 37, 5)]):
        X, y, beta = datasets.covtype_like(seed=seed, n=n_rows, n_cont=6, n_bin=4)
        n, p = X.shape
        dx = torch.as_tensor(X, device="cuda").contiguous()
        dy = torch.as_tensor(y, device="cuda").contiguous()
        z = torch.as_tensor((beta[None, :] + 0.3 * rng.standard_normal((C, p))).astype(np.float32), device="cuda")
        pe = torch.full((C,), float("nan"), dtype=torch.float64, device="cuda")
        g = torch.full((C, p), float("nan"), dtype=torch.float32, device="cuda")
        status = lib.gbn_logreg_potential_noalloc(stream, _ptr(dx), _ptr(dy), n, p, 1.0, _ptr(z), C, _ptr(pe),
                                                  _ptr(g))
        assert status == 0, lib.gbn_noalloc_last_error()
        ref_kernel = NUTS(models.LogisticRegression(X, y), num_chains=C, precision="fp32")
        pe_ref, g_ref = ref_kernel.potential_and_grad(z)
        torch.cuda.synchronize()
        ref_kernel.close()
        pe, g, pe_ref, g_ref, zh = (t.cpu().numpy() for t in (pe, g, pe_ref, g_ref, z))
        np.testing.assert_allclose(pe, pe_ref, rtol=2e-6, err_msg="call %d vs gbn_potential_and_grad" % call)
        scale = np.max(np.abs(g_ref), axis=1, keepdims=True)
        assert np.max(np.abs(g - g_ref) / np.maximum(scale, 1.0)) < 1e-3, "call %d" % call
        # FP64 oracle (numpyro's potential_energy of the covtype model, restated)
        X64, y64 = X.astype(np.float64), y.astype(np.float64)
        for c in range(C):
            pr = PR.logreg_potential(zh[c].astype(np.float64), X64, y64)
            gr = PR.logreg_grad(zh[c].astype(np.float64), X64, y64)
            assert abs(pe[c] - pr) <= 2e-6 * abs(pr) + 1e-4, (call, c, pe[c], pr)
            assert np.max(np.abs(g[c] - gr)) <= 1e-3 * max(np.max(np.abs(gr)), 1.0), (call, c)


@pytest.mark.gpu
def test_noalloc_rejects_bad_sizes_and_prior_scale():
    from numpyro_gb300 import _lib

    lib = _lib.load()
    d = torch.zeros(8, device="cuda")
    too_many = _lib.NOALLOC_MAX_POINTS + 1
    status = lib.gbn_logreg_potential_noalloc(None, _ptr(d), _ptr(d), 2, 2, 1.0, _ptr(d), too_many, _ptr(d),
                                              _ptr(d))
    assert status == 1
    assert b"GBN_NOALLOC_MAX_POINTS" in lib.gbn_noalloc_last_error()
    for bad in (0.0, -1.0, float("nan"), float("inf")):
        status = lib.gbn_logreg_potential_noalloc(None, _ptr(d), _ptr(d), 2, 2, bad, _ptr(d), 1, _ptr(d), _ptr(d))
        assert status == 1, bad
        assert b"prior_scale" in lib.gbn_noalloc_last_error()
