"""HMC and NUTS MCMCKernels backed by the GB300 engine (libgbnuts).

Mirrors numpyro/infer/hmc.py: ``HMCState`` has the same 13 fields in the same
order (hmc.py:31-47), ``HMCAdaptState`` the same 8 (hmc_util.py:18-30);
``HMC.__init__`` and ``NUTS.__init__`` take numpyro's arguments
(hmc.py:625-686, :916-951).  Fields are CUDA tensors batched over chains on
the leading axis, as numpyro's vectorized init produces them (hmc.py:796).

The ``model`` argument is a registry model (numpyro_gb300.models); arbitrary
Python potentials are rejected with NotImplementedError -- the engine has no
CPU or autodiff fallback.
"""
from collections import namedtuple
import ctypes
import math
import warnings

import numpy as np

from . import _lib
from .mcmc import MCMCKernel
from .models import Model

HMCState = namedtuple(
    "HMCState",
    ["i", "z", "z_grad", "potential_energy", "energy", "r", "trajectory_length", "num_steps",
     "accept_prob", "mean_accept_prob", "diverging", "adapt_state", "rng_key"],
)
HMCAdaptState = namedtuple(
    "HMCAdaptState",
    ["step_size", "inverse_mass_matrix", "mass_matrix_sqrt", "mass_matrix_sqrt_inv", "ss_state", "mm_state",
     "window_idx", "rng_key"],
)


def init_to_uniform(site=None, radius=2):
    """numpyro/infer/initialization.py:95 -- the only strategy the engine runs on device."""
    return init_to_uniform


def _torch():
    import torch

    return torch


def seed_from_key(rng_key):
    """Accepts an int seed, a (2,) uint32 key, or a (C, 2) batch of keys."""
    if isinstance(rng_key, (int, np.integer)):
        return int(rng_key) & 0xFFFFFFFFFFFFFFFF, None
    a = np.asarray(rng_key)
    if a.ndim == 0:
        return int(a) & 0xFFFFFFFFFFFFFFFF, None
    if a.ndim == 1:
        a = a.astype(np.uint64)
        return int((a[0] << np.uint64(32)) | a[-1]) if a.size > 1 else int(a[0]), None
    first = a[0].astype(np.uint64)
    return int((first[0] << np.uint64(32)) | first[-1]), a.shape[0]


def _ptr(t, ctype):
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctype)



def mass_blocks_of(model, dense_mass):
    """numpyro's block-structured dense_mass (a list of tuples of site names,
    numpyro/infer/hmc_util.py:439-486: each tuple a dense block over its sites, the sites in no
    tuple one diagonal block) as the engine's per-coordinate block ids: the tuple's index for its
    sites' coordinates, -1 for the rest."""
    slices = model.site_slices()
    blocks = np.full(model.latent_dim, -1, np.int32)
    seen = set()
    for b, names in enumerate(dense_mass):
        if isinstance(names, str) or not isinstance(names, (tuple, list)):
            raise ValueError("dense_mass blocks must be tuples of site names, got %r" % (names,))
        for name in names:
            if name not in slices:
                raise ValueError("dense_mass names site %r, which the model does not have (%s)"
                                 % (name, ", ".join(sorted(slices))))
            if name in seen:
                raise ValueError("site %r is in more than one dense_mass block" % (name,))
            seen.add(name)
            a, e, _ = slices[name]
            blocks[a:e] = b
    return blocks

class HMC(MCMCKernel):
    """Hamiltonian Monte Carlo with fixed trajectory length (numpyro/infer/hmc.py:541-822).

    Extra keyword-only arguments beyond numpyro's:
      engine: "fused" (per-chain trees, no lock-step; one persistent launch for the hierarchical
              family), "ticks" (per-chain trees, one launch per leapfrog step) or "plain"
              (lock-step, numpyro vmap semantics)
      precision: "fp32" or "bf16x3" (tensor-core logistic potential)
      num_chains: chains to run when ``init`` gets a single key
    """

    def __init__(self, model=None, potential_fn=None, kinetic_fn=None, step_size=1.0, inverse_mass_matrix=None,
                 adapt_step_size=True, adapt_mass_matrix=True, dense_mass=False, target_accept_prob=0.8,
                 num_steps=None, trajectory_length=2 * math.pi, init_strategy=init_to_uniform,
                 find_heuristic_step_size=False, forward_mode_differentiation=False, regularize_mass_matrix=True,
                 *, engine="fused", precision="fp32", num_chains=None, first_chain=0):
        if not (model is None) ^ (potential_fn is None):
            raise ValueError("Only one of `model` or `potential_fn` must be specified.")
        if potential_fn is not None:
            raise NotImplementedError(
                "the GB300 engine evaluates registry potentials only; pass model=<numpyro_gb300.models model>")
        if not isinstance(model, Model):
            raise NotImplementedError("model must be a numpyro_gb300.models registry model")
        if kinetic_fn is not None:
            raise NotImplementedError("only the Euclidean kinetic energy is supported")
        self._mass_blocks = None
        if isinstance(dense_mass, list) and dense_mass:
            self._mass_blocks = mass_blocks_of(model, dense_mass)
            dense_mass = True
        elif dense_mass not in (False, True, [], None):
            raise ValueError("dense_mass must be a bool or a list of tuples of site names")
        if init_strategy is not init_to_uniform:
            raise NotImplementedError("only init_to_uniform(radius=2) runs on the device")
        if type(self) is HMC:
            if num_steps is None and trajectory_length is None:
                raise ValueError("At least one of `num_steps` or `trajectory_length` must be specified.")
            if adapt_step_size and num_steps is not None and trajectory_length is not None:
                warnings.warn("If both `num_steps` and `trajectory_length` are specified step size can't be adapted")
        if engine not in ("fused", "plain", "ticks"):
            raise ValueError("engine must be 'fused', 'plain' or 'ticks'")
        if precision not in ("fp32", "bf16x3"):
            raise ValueError("precision must be 'fp32' or 'bf16x3'")
        self._model = model
        self._step_size = float(step_size)
        self._inverse_mass_matrix = inverse_mass_matrix
        self._adapt_step_size = adapt_step_size
        self._adapt_mass_matrix = adapt_mass_matrix
        self._dense_mass = bool(dense_mass)
        self._target_accept_prob = target_accept_prob
        self._num_steps = num_steps
        self._trajectory_length = None if trajectory_length is None else float(trajectory_length)
        self._algo = "HMC"
        self._max_tree_depth = 10
        self._init_strategy = init_strategy
        self._find_heuristic_step_size = find_heuristic_step_size
        self._forward_mode_differentiation = forward_mode_differentiation
        self._regularize_mass_matrix = regularize_mass_matrix
        self._engine = engine
        self._precision = precision
        self._num_chains = num_chains
        # global id of this kernel's chain 0: a run split over kernels (or GPUs), one seed and a
        # chain range each, gives every chain the draws it has in one kernel of all the chains
        if int(first_chain) < 0:
            raise ValueError("first_chain must be >= 0")
        self._first_chain = int(first_chain)
        self._handle = None
        self._handle_key = None
        self._keep = None
        self._num_warmup = 0
        self._seed = 0

    # ------------------------------------------------------------------ properties
    @property
    def model(self):
        return self._model

    @property
    def sample_field(self):
        return "z"

    @property
    def default_fields(self):
        return ("z", "diverging")

    def get_diagnostics_str(self, state):
        return "{} steps of size {:.2e}. acc. prob={:.2f}".format(
            int(state.num_steps.float().mean()), float(state.adapt_state.step_size.float().mean()),
            float(state.mean_accept_prob.float().mean()))

    def postprocess_fn(self, args, kwargs):
        return self._model.postprocess

    # ------------------------------------------------------------------ engine
    def _config(self, num_chains, seed):
        cfg = _lib.Config()
        cfg.num_chains = num_chains
        m = self._model
        cfg.chains_per_model = num_chains // getattr(m, "num_models", 1) if hasattr(m, "num_models") else 0
        cfg.algo = _lib.ALGO_NUTS if self._algo == "NUTS" else _lib.ALGO_HMC
        cfg.engine = {"fused": _lib.ENGINE_FUSED, "plain": _lib.ENGINE_PLAIN, "ticks": _lib.ENGINE_TICKS}[self._engine]
        cfg.precision = _lib.PREC_BF16X3 if self._precision == "bf16x3" else _lib.PREC_FP32
        mtd = self._max_tree_depth
        if isinstance(mtd, tuple):
            cfg.max_tree_depth_warmup, cfg.max_tree_depth = int(mtd[0]), int(mtd[1])
        else:
            cfg.max_tree_depth_warmup = cfg.max_tree_depth = int(mtd)
        cfg.adapt_step_size = int(bool(self._adapt_step_size))
        cfg.adapt_mass_matrix = int(bool(self._adapt_mass_matrix))
        cfg.dense_mass = int(self._dense_mass)
        if self._mass_blocks is not None:
            cfg.mass_blocks = self._mass_blocks.ctypes.data_as(_lib.c_int32_p)  # read at gbn_create
        cfg.regularize_mass_matrix = int(bool(self._regularize_mass_matrix))
        cfg.find_heuristic_step_size = int(bool(self._find_heuristic_step_size))
        cfg.num_steps = int(self._num_steps or 0)
        cfg.target_accept_prob = float(self._target_accept_prob)
        cfg.trajectory_length = float(self._trajectory_length) if self._trajectory_length is not None else -1.0
        cfg.max_delta_energy = 1000.0
        cfg.init_step_size = self._step_size
        cfg.seed = seed
        cfg.first_chain = self._first_chain
        return cfg

    def _ensure_handle(self, num_chains, seed):
        key = (num_chains, seed)
        if self._handle is not None and self._handle_key == key:
            return self._handle
        self.close()
        lib = _lib.load()
        desc, keep = self._model.descriptor()
        cfg = self._config(num_chains, seed)
        h = ctypes.c_void_p()
        _lib.check(lib.gbn_create(ctypes.byref(h), ctypes.byref(desc), ctypes.byref(cfg)))
        self._handle = h
        self._handle_key = key
        self._keep = keep
        return h

    def close(self):
        if self._handle is not None:
            _lib.load().gbn_destroy(self._handle)
            self._handle = None
            self._handle_key = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tuning(self):
        """Launch shapes the autotuner chose for this kernel's potential (gbn_tuning)."""
        if self._handle is None:
            return ""
        v = _lib.load().gbn_tuning(self._handle)
        return v.decode() if v else ""

    @property
    def num_chains(self):
        return self._handle_key[0] if self._handle_key else None

    @property
    def latent_dim(self):
        return self._model.latent_dim

    def _alloc_state(self, C, D):
        torch = _torch()
        dev = torch.device("cuda")
        f32 = dict(dtype=torch.float32, device=dev)
        f64 = dict(dtype=torch.float64, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        mshape = (C, D, D) if self._dense_mass else (C, D)  # HMCAdaptState mass matrices, vmapped
        adapt = HMCAdaptState(
            torch.zeros(C, **f32), torch.zeros(mshape, **f32), torch.zeros(mshape, **f32), torch.zeros(mshape, **f32),
            torch.zeros(C, 5, **f64),
            (torch.zeros(C, D, **f64), torch.zeros(mshape, **f64), torch.zeros(C, **i32)),
            torch.zeros(C, **i32), torch.zeros(C, 2, dtype=torch.int32, device=dev))
        traj = self._trajectory_length if self._algo == "HMC" else None
        return HMCState(
            torch.zeros(C, **i32), torch.zeros(C, D, **f32), torch.zeros(C, D, **f32), torch.zeros(C, **f64),
            torch.zeros(C, **f64), None, traj, torch.zeros(C, **i32), torch.zeros(C, **f32), torch.zeros(C, **f32),
            torch.zeros(C, dtype=torch.uint8, device=dev), adapt, adapt.rng_key)

    @staticmethod
    def _cstate(state):
        a = state.adapt_state
        st = _lib.State()
        st.i = _ptr(state.i, _lib.c_int32_p)
        st.z = _ptr(state.z, _lib.c_float_p)
        st.z_grad = _ptr(state.z_grad, _lib.c_float_p)
        st.potential_energy = _ptr(state.potential_energy, _lib.c_double_p)
        st.energy = _ptr(state.energy, _lib.c_double_p)
        st.num_steps = _ptr(state.num_steps, _lib.c_int32_p)
        st.accept_prob = _ptr(state.accept_prob, _lib.c_float_p)
        st.mean_accept_prob = _ptr(state.mean_accept_prob, _lib.c_float_p)
        st.diverging = _ptr(state.diverging, _lib.c_uint8_p)
        st.step_size = _ptr(a.step_size, _lib.c_float_p)
        st.inverse_mass_matrix = _ptr(a.inverse_mass_matrix, _lib.c_float_p)
        st.mass_matrix_sqrt = _ptr(a.mass_matrix_sqrt, _lib.c_float_p)
        st.mass_matrix_sqrt_inv = _ptr(a.mass_matrix_sqrt_inv, _lib.c_float_p)
        st.ss_state = _ptr(a.ss_state, _lib.c_double_p)
        st.mm_mean = _ptr(a.mm_state[0], _lib.c_double_p)
        st.mm_m2 = _ptr(a.mm_state[1], _lib.c_double_p)
        st.mm_n = _ptr(a.mm_state[2], _lib.c_int32_p)
        st.window_idx = _ptr(a.window_idx, _lib.c_int32_p)
        st.rng_key = _ptr(state.rng_key, _lib.c_uint32_p)
        return st

    @staticmethod
    def copy_state(state):
        def cp(x):
            if x is None or isinstance(x, (int, float)):
                return x
            if isinstance(x, tuple):
                return type(x)(*[cp(v) for v in x]) if hasattr(x, "_fields") else tuple(cp(v) for v in x)
            return x.clone()

        adapt = cp(state.adapt_state)
        out = HMCState(*[cp(v) for v in state[:11]], adapt, None)
        return out._replace(rng_key=adapt.rng_key)

    def _stream(self):
        torch = _torch()
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    # ------------------------------------------------------------------ MCMCKernel API
    def init(self, rng_key, num_warmup, init_params=None, model_args=(), model_kwargs={}):
        """HMC.init (hmc.py:740-799): vectorized over chains.

        rng_key: int seed, a (2,) key (num_chains from the constructor) or a
        (C, 2) batch of keys (C chains).  init_params: optional [C, D] array of
        unconstrained initial values."""
        torch = _torch()
        seed, nkeys = seed_from_key(rng_key)
        C = nkeys or self._num_chains or 1
        h = self._ensure_handle(C, seed)
        D = self._model.latent_dim
        self._num_warmup = int(num_warmup)
        self._seed = seed
        state = self._alloc_state(C, D)
        z0 = None
        if init_params is not None:
            z0 = torch.as_tensor(np.asarray(init_params, np.float32).reshape(C, D), device="cuda").contiguous()
        inv0 = None
        if self._inverse_mass_matrix is not None:
            inv = np.asarray(self._inverse_mass_matrix, np.float32)
            if self._dense_mass:
                if inv.shape[-1:] == (D,) and (inv.ndim == 1 or inv.shape[-2:] != (D, D)):
                    inv = np.apply_along_axis(np.diag, -1, inv)  # a diagonal given for a dense kernel
                inv = np.broadcast_to(inv, (C, D, D))
            else:
                if inv.ndim >= 2 and inv.shape[-2:] == (D, D):
                    inv = np.diagonal(inv, axis1=-2, axis2=-1)
                inv = np.broadcast_to(inv, (C, D))
            inv0 = torch.as_tensor(np.ascontiguousarray(inv), device="cuda")
        st = self._cstate(state)
        lib = _lib.load()
        _lib.check(lib.gbn_init(h, self._stream(), int(num_warmup),
                                ctypes.c_void_p(z0.data_ptr()) if z0 is not None else None,
                                ctypes.c_void_p(inv0.data_ptr()) if inv0 is not None else None,
                                ctypes.byref(st)), h)
        torch.cuda.current_stream().synchronize()
        return state

    def sample(self, state, model_args=(), model_kwargs={}):
        """One transition for every chain (hmc.py:459-530); the input state is not modified."""
        new = self.copy_state(state)
        st = self._cstate(new)
        lib = _lib.load()
        _lib.check(lib.gbn_sample(self._handle, self._stream(), ctypes.byref(st)), self._handle)
        return new

    def sample_async(self, state, model_args=(), model_kwargs={}):
        """``sample`` enqueued on the current stream without any host synchronisation
        (gbn_sample_async): the tick loop runs on the device.  Bit-identical to ``sample``;
        ``check_async`` reports a tick budget exhausted on the device."""
        new = self.copy_state(state)
        st = self._cstate(new)
        _lib.check(_lib.load().gbn_sample_async(self._handle, self._stream(), ctypes.byref(st)), self._handle)
        return new

    def check_async(self):
        """Waits for the current stream and raises if an asynchronous transition failed on the device."""
        _lib.check(_lib.load().gbn_check_async(self._handle, self._stream()), self._handle)

    def run_device(self, state, num_iterations, collect_start=0, thinning=1, collect=("z",)):
        """Runs ``num_iterations`` transitions per chain entirely on the device,
        updating ``state`` in place; returns a dict of collected [C, S, ...] tensors."""
        torch = _torch()
        C, D = state.z.shape
        S = max(0, (num_iterations - collect_start + thinning - 1) // thinning) if collect_start < num_iterations else 0
        out = {}
        col = _lib.Collect()
        dev = state.z.device
        if S > 0:
            if "z" in collect:
                out["z"] = torch.zeros(C, S, D, dtype=torch.float32, device=dev)
                col.samples = _ptr(out["z"], _lib.c_float_p)
            if "num_steps" in collect:
                out["num_steps"] = torch.empty(C, S, dtype=torch.int32, device=dev)
                col.num_steps = _ptr(out["num_steps"], _lib.c_int32_p)
            if "accept_prob" in collect:
                out["accept_prob"] = torch.empty(C, S, dtype=torch.float32, device=dev)
                col.accept_prob = _ptr(out["accept_prob"], _lib.c_float_p)
            if "diverging" in collect:
                out["diverging"] = torch.empty(C, S, dtype=torch.uint8, device=dev)
                col.diverging = _ptr(out["diverging"], _lib.c_uint8_p)
            if "potential_energy" in collect:
                out["potential_energy"] = torch.empty(C, S, dtype=torch.float64, device=dev)
                col.potential_energy = _ptr(out["potential_energy"], _lib.c_double_p)
            if "adapt_state.step_size" in collect:
                out["adapt_state.step_size"] = torch.empty(C, S, dtype=torch.float32, device=dev)
                col.step_size = _ptr(out["adapt_state.step_size"], _lib.c_float_p)
        st = self._cstate(state)
        lib = _lib.load()
        _lib.check(lib.gbn_run(self._handle, self._stream(), ctypes.byref(st), int(num_iterations),
                               int(collect_start), int(thinning), ctypes.byref(col)), self._handle)
        return out

    def stats(self):
        s = _lib.Stats()
        _lib.check(_lib.load().gbn_get_stats(self._handle, ctypes.byref(s)), self._handle)
        return {"ticks": s.ticks, "potential_launches": s.potential_launches, "device_ms": s.device_ms}

    def potential_and_grad(self, z):
        """U(z) and dU/dz for a [K, D] CUDA tensor of latent points."""
        torch = _torch()
        z = z.to(device="cuda", dtype=torch.float32).contiguous()
        K = z.shape[0]
        if self._handle is None:
            self._ensure_handle(K, self._seed)
        pe = torch.empty(K, dtype=torch.float64, device=z.device)
        g = torch.empty_like(z)
        _lib.check(_lib.load().gbn_potential_and_grad(self._handle, self._stream(), ctypes.c_void_p(z.data_ptr()),
                                                      K, ctypes.c_void_p(pe.data_ptr()),
                                                      ctypes.c_void_p(g.data_ptr())), self._handle)
        return pe, g

    def __getstate__(self):
        state = self.__dict__.copy()
        state["_handle"] = None
        state["_handle_key"] = None
        state["_keep"] = None
        return state


class NUTS(HMC):
    """No-U-Turn Sampler (numpyro/infer/hmc.py:825-951)."""

    def __init__(self, model=None, potential_fn=None, kinetic_fn=None, step_size=1.0, inverse_mass_matrix=None,
                 adapt_step_size=True, adapt_mass_matrix=True, dense_mass=False, target_accept_prob=0.8,
                 trajectory_length=None, max_tree_depth=10, init_strategy=init_to_uniform,
                 find_heuristic_step_size=False, forward_mode_differentiation=False, regularize_mass_matrix=True,
                 *, engine="fused", precision="fp32", num_chains=None, first_chain=0):
        super().__init__(model=model, potential_fn=potential_fn, kinetic_fn=kinetic_fn, step_size=step_size,
                         inverse_mass_matrix=inverse_mass_matrix, adapt_step_size=adapt_step_size,
                         adapt_mass_matrix=adapt_mass_matrix, dense_mass=dense_mass,
                         target_accept_prob=target_accept_prob, trajectory_length=trajectory_length,
                         init_strategy=init_strategy, find_heuristic_step_size=find_heuristic_step_size,
                         forward_mode_differentiation=forward_mode_differentiation,
                         regularize_mass_matrix=regularize_mass_matrix, engine=engine, precision=precision,
                         num_chains=num_chains, first_chain=first_chain)
        self._max_tree_depth = max_tree_depth
        self._algo = "NUTS"


def hmc(potential_fn=None, kinetic_fn=None, algo="NUTS", *, engine="fused", precision="fp32", num_chains=None):
    """The functional API (numpyro/infer/hmc.py:113-538): returns ``(init_kernel, sample_kernel)``.

    ``potential_fn`` is a registry model (numpyro_gb300.models), passed where numpyro takes the
    traced ``model_info.potential_fn``; any other callable raises NotImplementedError, as the
    kernel classes do.  ``init_kernel`` takes numpyro's arguments (hmc.py:193-212) and builds the
    NUTS or HMC kernel that ``sample_kernel`` then steps (hmc.py:459-530).  ``init_params`` is
    None (init_to_uniform on the device), an array of unconstrained values ([D] or [C, D]) or an
    object with a ``.z`` array such as numpyro's ParamInfo.  ``rng_key`` is an int seed, a key or
    a [C, 2] batch of keys; C chains run vectorized, one when a single key is given and
    ``num_chains`` is None.
    """
    if algo not in ("HMC", "NUTS"):
        raise ValueError("`algo` must be one of `HMC` or `NUTS`.")
    if potential_fn is None:
        raise ValueError("potential_fn (a numpyro_gb300.models registry model) is required")
    if not isinstance(potential_fn, Model):
        raise NotImplementedError(
            "the GB300 engine evaluates registry potentials only; pass a numpyro_gb300.models model")
    if kinetic_fn is not None:
        raise NotImplementedError("only the Euclidean kinetic energy is supported")
    model = potential_fn
    holder = {}

    def init_kernel(init_params, num_warmup, step_size=1.0, inverse_mass_matrix=None, adapt_step_size=True,
                    adapt_mass_matrix=True, dense_mass=False, target_accept_prob=0.8, *, num_steps=None,
                    trajectory_length=2 * math.pi, max_tree_depth=10, find_heuristic_step_size=False,
                    forward_mode_differentiation=False, regularize_mass_matrix=True, model_args=(),
                    model_kwargs=None, rng_key=None):
        common = dict(model=model, step_size=step_size, inverse_mass_matrix=inverse_mass_matrix,
                      adapt_step_size=adapt_step_size, adapt_mass_matrix=adapt_mass_matrix, dense_mass=dense_mass,
                      target_accept_prob=target_accept_prob, find_heuristic_step_size=find_heuristic_step_size,
                      forward_mode_differentiation=forward_mode_differentiation,
                      regularize_mass_matrix=regularize_mass_matrix, engine=engine, precision=precision,
                      num_chains=num_chains)
        if algo == "NUTS":
            kernel = NUTS(max_tree_depth=max_tree_depth, **common)
        else:
            kernel = HMC(num_steps=num_steps, trajectory_length=trajectory_length, **common)
        old = holder.pop("kernel", None)
        if old is not None:
            old.close()
        holder["kernel"] = kernel
        key = 0 if rng_key is None else rng_key
        z0 = getattr(init_params, "z", init_params)
        if z0 is not None:
            z0 = np.asarray(z0.detach().cpu() if hasattr(z0, "detach") else z0, np.float32)
            if z0.ndim == 1:  # one starting point for every chain
                C = seed_from_key(key)[1] or num_chains or 1
                z0 = np.broadcast_to(z0, (C, z0.shape[0]))
        return kernel.init(key, num_warmup, z0)

    def sample_kernel(hmc_state, model_args=(), model_kwargs=None):
        if "kernel" not in holder:
            raise RuntimeError("call init_kernel before sample_kernel")
        return holder["kernel"].sample(hmc_state)

    init_kernel.kernel = lambda: holder.get("kernel")  # the kernel object behind the closures
    return init_kernel, sample_kernel
