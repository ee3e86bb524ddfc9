"""Host pieces of numpyro's functional API: fori_collect (numpyro/util.py) and initialize_model
(numpyro/infer/util.py)."""
from collections import namedtuple

import numpy as np


def _is_namedtuple(x):
    return isinstance(x, tuple) and hasattr(x, "_fields")


def _tree_map(fn, x):
    if x is None:
        return None
    if isinstance(x, dict):
        return {k: _tree_map(fn, v) for k, v in x.items()}
    if _is_namedtuple(x):
        return type(x)(*[_tree_map(fn, v) for v in x])
    if isinstance(x, (tuple, list)):
        return type(x)(_tree_map(fn, v) for v in x)
    return fn(x)


def _tree_set(collection, idx, value):
    if collection is None:
        return
    if isinstance(collection, dict):
        for k in collection:
            _tree_set(collection[k], idx, value[k])
    elif isinstance(collection, (tuple, list)):
        for c, v in zip(collection, value):
            _tree_set(c, idx, v)
    else:
        collection[idx] = _to_host(value)


def _to_host(x):
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def fori_collect(lower, upper, body_fun, init_val, transform=lambda x: x, progbar=False, progress_rate=None,
                 return_last_val=False, collection_size=None, thinning=1, **progbar_opts):
    """numpyro.util.fori_collect (numpyro/util.py:321-454) as a host loop.

    Runs ``body_fun`` ``upper`` times from ``init_val`` and collects ``transform(val)`` into host
    arrays with a leading axis of ``(upper - lower) // thinning`` (or ``collection_size``; the
    entries past the collected ones stay zero).  Iteration i writes slot
    ``(i - start) // thinning`` when that is >= 0, with ``start = lower + (upper - lower) % thinning``,
    so each slot keeps the last value of its group of ``thinning`` iterations, as in the
    reference.  The body runs as its own launches (for instance one NUTS transition per call);
    ``MCMC.run`` keeps the whole loop on the device.  The progress-bar arguments are accepted and
    ignored.
    """
    assert lower <= upper
    assert thinning >= 1
    size = (upper - lower) // thinning if collection_size is None else collection_size
    assert size >= (upper - lower) // thinning
    start = lower + (upper - lower) % thinning
    template = _tree_map(_to_host, transform(init_val))
    collection = _tree_map(lambda x: np.zeros((size,) + x.shape, x.dtype), template)
    val = init_val
    for i in range(upper):
        val = body_fun(val)
        idx = (i - start) // thinning
        if idx >= 0:
            _tree_set(collection, idx, transform(val))
    return (collection, val) if return_last_val else collection


# numpyro/infer/util.py:47-50
ModelInfo = namedtuple("ModelInfo", ["param_info", "potential_fn", "postprocess_fn", "model_trace"])
ParamInfo = namedtuple("ParamInfo", ["z", "potential_energy", "z_grad"])


def initialize_model(rng_key, model, *, init_strategy=None, dynamic_args=False, model_args=(), model_kwargs=None,
                     forward_mode_differentiation=False, validate_grad=True):
    """numpyro.infer.util.initialize_model (numpyro/infer/util.py:663) for a registry model.

    Returns ``ModelInfo(param_info, potential_fn, postprocess_fn, model_trace)`` for the functional
    API: ``potential_fn`` is the model itself (what ``hmc`` takes), ``postprocess_fn`` maps
    unconstrained [..., D] values to the constrained sites, and ``param_info.z`` is None, which
    makes ``init_kernel`` draw init_to_uniform(radius=2) starting points on the device with the
    reference's retries (numpyro/infer/util.py:366-508).  There is no model trace (None).
    """
    from .hmc import init_to_uniform
    from .models import Model

    if not isinstance(model, Model):
        raise NotImplementedError("the GB300 engine runs registry models only (numpyro_gb300.models)")
    if init_strategy is not None and init_strategy is not init_to_uniform:
        raise NotImplementedError("only init_to_uniform(radius=2) runs on the device")
    if dynamic_args:
        raise NotImplementedError("registry models carry their data; dynamic_args is not supported")
    return ModelInfo(ParamInfo(None, None, None), model, model.postprocess, None)
