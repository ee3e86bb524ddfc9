"""MCMCKernel interface and the MCMC driver (numpyro/infer/mcmc.py).

``MCMCKernel`` restates the plugin ABC (mcmc.py:33-159).  ``MCMC`` restates
the driver's public surface -- run / warmup / get_samples / get_extra_fields /
print_summary / post_warmup_state / last_state / transfer_states_to_host
(mcmc.py:225-809) -- for
``chain_method="vectorized"``.  With a GB300 kernel (numpyro_gb300.HMC/NUTS)
the whole warmup+sampling loop runs on the device in one gbn_run call (the
analogue of fori_collect's single compiled loop, numpyro/util.py:321-454);
any other MCMCKernel is driven by a Python loop over ``kernel.sample``.
"""
from abc import ABC, abstractmethod
from operator import attrgetter
import warnings

import numpy as np

from . import diagnostics


class MCMCKernel(ABC):
    """Markov transition kernel interface (numpyro/infer/mcmc.py:33-159)."""

    def postprocess_fn(self, model_args, model_kwargs):
        return lambda x: x

    @abstractmethod
    def init(self, rng_key, num_warmup, init_params, model_args, model_kwargs):
        raise NotImplementedError

    @abstractmethod
    def sample(self, state, model_args, model_kwargs):
        raise NotImplementedError

    @property
    def sample_field(self):
        raise NotImplementedError

    @property
    def default_fields(self):
        return (self.sample_field,)

    @property
    def is_ensemble_kernel(self):
        return False

    def get_diagnostics_str(self, state):
        return ""


def _nested_get(state, name):
    return attrgetter(name)(state)


def _to_numpy(x):
    if hasattr(x, "detach"):
        return x.detach().cpu().numpy()
    return np.asarray(x)


class MCMC:
    """MCMC driver with numpyro's constructor (numpyro/infer/mcmc.py:326-393)."""

    def __init__(self, sampler, *, num_warmup, num_samples, num_chains=1, thinning=1, postprocess_fn=None,
                 chain_method="vectorized", progress_bar=False, progress_rate=None, jit_model_args=False,
                 keep_on_device=False):
        """keep_on_device (no counterpart in numpyro's constructor): with a GB300 kernel, leave the
        collected draws in HBM as torch tensors, as numpyro leaves them on the accelerator until
        transfer_states_to_host (mcmc.py:799-804); print_summary then computes its statistics on the
        device (device_diagnostics) and only the per-coordinate results move."""
        self.keep_on_device = bool(keep_on_device)
        self.sampler = sampler
        self._sample_field = sampler.sample_field
        self._default_fields = sampler.default_fields
        self.num_warmup = num_warmup
        self.num_samples = num_samples
        self.num_chains = num_chains
        if not isinstance(thinning, int) or thinning < 1:
            raise ValueError("thinning must be a positive integer")
        self.thinning = thinning
        self.postprocess_fn = postprocess_fn
        if not callable(chain_method) and chain_method not in ["parallel", "vectorized", "sequential"]:
            raise ValueError('Only supporting the following methods to draw chains: "sequential", "parallel", '
                             'or "vectorized"')
        if chain_method != "vectorized" and num_chains > 1:
            warnings.warn("the GB300 engine runs every chain on one GPU; chain_method=%r is executed as "
                          "'vectorized' (per-chain results are identical)" % (chain_method,))
        self.chain_method = chain_method
        self.progress_bar = progress_bar
        self.progress_rate = progress_rate
        self._jit_model_args = jit_model_args
        self._states = None
        self._states_flat = None
        self._last_state = None
        self._warmup_state = None
        self.timing = {}

    @property
    def post_warmup_state(self):
        return self._warmup_state

    @post_warmup_state.setter
    def post_warmup_state(self, state):
        self._warmup_state = state

    @property
    def last_state(self):
        return self._last_state

    def _is_device_kernel(self):
        from .hmc import HMC

        return isinstance(self.sampler, HMC)

    def _collect_fields(self, extra_fields):
        fields, remove = {}, []
        for f in (self._sample_field,) + tuple(self._default_fields) + tuple(extra_fields):
            if f.startswith("~%s." % self._sample_field):
                remove.append(f[len(self._sample_field) + 2:])
            else:
                fields[f] = None
        return tuple(fields), tuple(remove)

    def warmup(self, rng_key, *args, extra_fields=(), collect_warmup=False, init_params=None, **kwargs):
        """Warmup only; stores post_warmup_state (mcmc.py:589-633)."""
        self._warmup_state = None
        self._run(rng_key, args, kwargs, extra_fields, init_params, phase="warmup", collect_warmup=collect_warmup)
        self._warmup_state = self._last_state

    def run(self, rng_key, *args, extra_fields=(), init_params=None, **kwargs):
        """Run warmup (unless post_warmup_state is set) and sampling (mcmc.py:635-729)."""
        self._run(rng_key, args, kwargs, extra_fields, init_params)

    def _run(self, rng_key, args, kwargs, extra_fields, init_params, phase=None, collect_warmup=False):
        import time

        fields, remove = self._collect_fields(extra_fields)
        if phase == "warmup":
            n_iter = self.num_warmup
            lower = 0 if collect_warmup else n_iter
        elif self._warmup_state is not None:
            n_iter = self.num_samples
            lower = 0
        else:
            n_iter = self.num_warmup + self.num_samples
            lower = self.num_warmup
        t0 = time.perf_counter()
        if self._is_device_kernel():
            states, last = self._run_device(rng_key, args, kwargs, fields, init_params, n_iter, lower)
        else:
            states, last = self._run_python(rng_key, args, kwargs, fields, init_params, n_iter, lower)
        self.timing = {"wall_s": time.perf_counter() - t0}
        sample = states.pop(self._sample_field, None)
        if sample is not None:
            post = self.postprocess_fn or self.sampler.postprocess_fn(args, kwargs)
            sample = post(sample)
            if isinstance(sample, dict):
                for site in remove:
                    sample.pop(site, None)
            states = {self._sample_field: sample, **states}
        self._states = states
        self._states_flat = None
        self._last_state = last

    def _run_device(self, rng_key, args, kwargs, fields, init_params, n_iter, lower):
        import torch

        from .hmc import HMC, seed_from_key

        kernel = self.sampler
        if kernel._num_chains is None:
            kernel._num_chains = self.num_chains
        if self._warmup_state is not None:
            state = HMC.copy_state(self._warmup_state)
            seed, _ = seed_from_key(rng_key)
            kernel._ensure_handle(state.z.shape[0], kernel._handle_key[1] if kernel._handle_key else seed)
        else:
            state = kernel.init(rng_key, self.num_warmup, init_params, args, kwargs)
        dev_fields = []
        for f in fields:
            if f in ("z", "num_steps", "accept_prob", "diverging", "potential_energy", "adapt_state.step_size"):
                dev_fields.append(f)
            else:
                raise NotImplementedError("field %r cannot be collected by the device engine" % f)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        out = kernel.run_device(state, n_iter, collect_start=lower, thinning=self.thinning, collect=dev_fields)
        ev1.record()
        torch.cuda.synchronize()
        self.device_ms = ev0.elapsed_time(ev1)
        states = {}
        for f in fields:
            if f in out:
                if self.keep_on_device:
                    v = out[f].bool() if f == "diverging" else out[f]
                else:
                    v = _to_numpy(out[f])
                    if f == "diverging":
                        v = v.astype(bool)
                states[f] = v
            else:
                states[f] = np.zeros((state.z.shape[0], 0) + ((state.z.shape[1],) if f == "z" else ()))
        return states, state

    def _run_python(self, rng_key, args, kwargs, fields, init_params, n_iter, lower):
        kernel = self.sampler
        state = self._warmup_state if self._warmup_state is not None else kernel.init(
            rng_key, self.num_warmup, init_params, args, kwargs)
        collected = {f: [] for f in fields}
        for j in range(n_iter):
            state = kernel.sample(state, args, kwargs)
            if j >= lower and (j - lower) % self.thinning == 0:
                for f in fields:
                    collected[f].append(_to_numpy(_nested_get(state, f)))
        states = {}
        for f, v in collected.items():
            arr = np.stack(v, axis=0) if v else np.zeros((0,))
            if arr.ndim >= 2:
                arr = np.swapaxes(arr, 0, 1)  # (C, S, ...)
            states[f] = arr
        return states, state

    def _flat(self, x):
        return {k: self._flat(v) for k, v in x.items()} if isinstance(x, dict) else \
            x.reshape((x.shape[0] * x.shape[1],) + x.shape[2:])

    def get_samples(self, group_by_chain=False):
        """(mcmc.py:731-755)"""
        s = self._states[self._sample_field]
        return s if group_by_chain else self._flat(s)

    def get_extra_fields(self, group_by_chain=False):
        out = {k: v for k, v in self._states.items() if k != self._sample_field}
        return out if group_by_chain else {k: self._flat(v) for k, v in out.items()}

    def transfer_states_to_host(self):
        """Collected states as host arrays (mcmc.py:799-804).  The device run copies its draws to
        host memory once, at the end, unless keep_on_device; this converts anything still on the
        device.  last_state stays on the device, to resume from."""
        def conv(x):
            return {k: conv(v) for k, v in x.items()} if isinstance(x, dict) else _to_numpy(x)

        if self._states is not None:
            self._states = conv(self._states)
        self._states_flat = None

    def print_summary(self, prob=0.9, exclude_deterministic=True):
        """(mcmc.py:769-797)"""
        sites = self._states[self._sample_field]
        if isinstance(sites, dict) and exclude_deterministic:
            names = [s.name for s in getattr(getattr(self.sampler, "model", None), "sites", ())]
            if names:
                sites = {k: v for k, v in sites.items() if k in names}
        leaves = list(sites.values()) if isinstance(sites, dict) else [sites]
        if leaves and all(hasattr(v, "device") and hasattr(v, "detach") for v in leaves):
            from . import device_diagnostics

            diagnostics.print_stats(device_diagnostics.summary(sites, prob=prob))
        else:
            diagnostics.print_summary(sites, prob=prob)
        extra = self.get_extra_fields()
        if "diverging" in extra:
            d = extra["diverging"]
            print("Number of divergences: {}".format(int(d.sum().item() if hasattr(d, "device") else np.sum(d))))
