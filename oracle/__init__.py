"""CPU oracle for the NUTS/HMC hot path -- TEST INFRASTRUCTURE ONLY.

This package is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and its
``--impl reference`` arm) may import it.  The product path
(``numpyro_gb300``) never imports, links or executes anything in here; when
its CUDA library is missing it raises instead of falling back to this code.

Contents
--------
philox.py          Philox4x32-10 counter-based generator and the random-stream
                   address layout shared bit-for-bit with the CUDA kernels.
potentials_ref.py  FP64 closed-form potentials (negative log joint in the
                   unconstrained space, including log-det-Jacobians) and
                   their analytic gradients for the model registry.
nuts_ref.py        FP64 restatement of numpyro's HMC/NUTS transition,
                   iterative tree building, velocity Verlet, dual averaging,
                   Welford covariance and the warmup adapter.
nuts_ref.c         The same algorithm in C (FP64 or FP32 build, OpenMP over
                   chains): the timed CPU baseline and a fast parity oracle.

Parity pinning: numpyro itself cannot run here (it needs jax/jaxlib, which are
not installed and cannot be fetched).  The restatement is pinned against the
known answers held by numpyro's own tests (test/infer/test_hmc_util.py,
test/test_diagnostics.py) and against scipy.stats log-densities and central
finite differences; bit-level parity with JAX's threefry stream is not
pinnable and is not claimed.
"""
