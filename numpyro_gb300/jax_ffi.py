"""The jax side of the drop-in boundary: jax.ffi targets over libgbnuts.

numpyro calls ``MCMCKernel.sample`` inside ``jit`` (numpyro/infer/mcmc.py:188-190, fori_collect
numpyro/util.py:386-403) and differentiates ``potential_fn`` with ``value_and_grad``
(numpyro/infer/hmc_util.py:242-252).  Under jax those become XLA custom calls into the handlers
of ``csrc/xla_ffi.cc`` (built as ``libgbnuts_xla.so`` when the XLA FFI headers are available):

* ``potential_and_grad(kernel, z)`` -- U and dU/dz of a [K, D] batch (gbn_potential_and_grad);
* ``potential_fn(kernel)`` -- U as a ``jax.custom_vjp`` whose backward pass is the hand-written
  adjoint (gbn_potential_vjp semantics: the cotangent scales dU/dz), not autodiff;
* ``sample(kernel, leaves)`` -- one transition of every chain (gbn_sample_async: no host
  synchronisation, no allocation), the 19 state buffers aliased from input to output.

The handle travels as an integer attribute (``gbn_handle_id``).  U is float64: enable
``jax_enable_x64`` as numpyro's FP64 mode does.  jax is imported lazily and guarded:
``unavailable()`` says why the path cannot run (jax absent, or the handler library not built).
"""
import ctypes
import os

import numpy as np

from . import _lib

try:  # jax is optional: the torch and ctypes paths do not need it
    import jax
    import jax.numpy as jnp

    _JAX_ERROR = None
except ImportError as ex:  # pragma: no cover - depends on the environment
    jax = jnp = None
    _JAX_ERROR = str(ex)

XLA_LIB_PATH = os.path.join(os.path.dirname(_lib.LIB_PATH), "libgbnuts_xla.so")
TARGETS = ("gbn_xla_potential_and_grad", "gbn_xla_potential_vjp", "gbn_xla_sample")
# gbn_state field order (include/gbnuts.h), the argument and result order of gbn_xla_sample
STATE_FIELDS = ("i", "z", "z_grad", "potential_energy", "energy", "num_steps", "accept_prob", "mean_accept_prob",
                "diverging", "step_size", "inverse_mass_matrix", "mass_matrix_sqrt", "mass_matrix_sqrt_inv",
                "ss_state", "mm_mean", "mm_m2", "mm_n", "window_idx", "rng_key")

_registered = False


def unavailable():
    """None when the jax path can run, else the reason it cannot."""
    if jax is None:
        return "jax is not installed (%s)" % _JAX_ERROR
    if not os.path.exists(XLA_LIB_PATH):
        return "libgbnuts_xla.so is not built: the XLA FFI headers (jax.ffi.include_dir()) were not found at build time"
    return None


def register():
    """Registers the three FFI targets with XLA for the CUDA platform (once per process)."""
    global _registered
    why = unavailable()
    if why:
        raise RuntimeError("numpyro_gb300.jax_ffi: " + why)
    if _registered:
        return
    lib = ctypes.CDLL(XLA_LIB_PATH)
    for name in TARGETS:
        jax.ffi.register_ffi_target(name, jax.ffi.pycapsule(getattr(lib, name)), platform="CUDA")
    _registered = True


def handle_id(kernel):
    """Registry id of a NUTS/HMC kernel's library handle (the kernel must have been initialised)."""
    if kernel._handle is None:
        raise RuntimeError("the kernel has no library handle yet: call kernel.init first")
    return int(_lib.load().gbn_handle_id(kernel._handle))


def potential_and_grad(kernel, z):
    """U(z) (float64 [K]) and dU/dz (float32 [K, D]) through XLA for a [K, D] batch."""
    register()
    z = jnp.asarray(z, jnp.float32)
    out = (jax.ShapeDtypeStruct(z.shape[:1], jnp.float64), jax.ShapeDtypeStruct(z.shape, jnp.float32))
    return jax.ffi.ffi_call("gbn_xla_potential_and_grad", out)(z, handle=np.int64(handle_id(kernel)))


def potential_fn(kernel):
    """numpyro's ``potential_fn`` for a [K, D] batch as a ``jax.custom_vjp``: the forward pass is
    the fused potential, the backward pass the hand-written adjoint (cotangent x dU/dz)."""
    register()
    hid = np.int64(handle_id(kernel))

    def call(z):
        z = jnp.asarray(z, jnp.float32)
        out = (jax.ShapeDtypeStruct(z.shape[:1], jnp.float64), jax.ShapeDtypeStruct(z.shape, jnp.float32))
        return jax.ffi.ffi_call("gbn_xla_potential_and_grad", out)(z, handle=hid)

    @jax.custom_vjp
    def potential(z):
        return call(z)[0]

    def fwd(z):
        pe, grad = call(z)
        return pe, grad

    def bwd(grad, cot):
        return (cot.astype(grad.dtype)[:, None] * grad,)

    potential.defvjp(fwd, bwd)
    return potential


def sample(kernel, leaves):
    """One transition of every chain through XLA (gbn_sample_async).  ``leaves``: the 19 state
    arrays in ``STATE_FIELDS`` order (chains on the leading axis, dtypes of include/gbnuts.h);
    returns the new arrays, which XLA aliases to the inputs."""
    register()
    if len(leaves) != len(STATE_FIELDS):
        raise ValueError("expected %d state arrays (%s)" % (len(STATE_FIELDS), ", ".join(STATE_FIELDS)))
    out = tuple(jax.ShapeDtypeStruct(x.shape, x.dtype) for x in leaves)
    fn = jax.ffi.ffi_call("gbn_xla_sample", out, input_output_aliases={k: k for k in range(len(leaves))})
    return fn(*leaves, handle=np.int64(handle_id(kernel)))
