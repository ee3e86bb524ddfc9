"""Builds and loads the C oracle (test infrastructure / CPU baseline only).

Compiles oracle/nuts_ref.c twice (REAL=double, REAL=float) with gcc + OpenMP
into oracle/_build/.  No architecture-specific flags: the same source builds
on the x86 development container and the Arm GPU machine.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "nuts_ref.c")


def _lib_path(prec):
    return os.path.join(BUILD, "libnutsref_%s.so" % prec)


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    out = []
    for prec, real in (("f64", "double"), ("f32", "float")):
        path = _lib_path(prec)
        if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(SRC):
            # the FP32 build (timed CPU baseline) may reassociate sums so gcc vectorises the
            # dot products; NaN/inf semantics are kept (no -ffast-math)
            extra = ["-fassociative-math", "-fno-signed-zeros", "-fno-trapping-math"] if real == "float" else []
            cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=gnu11", "-DREAL=%s" % real,
                   "-DREAL_IS_FLOAT=%d" % (real == "float")] + extra + [SRC, "-o", path + ".tmp", "-lm"]
            subprocess.check_call(cmd)
            os.replace(path + ".tmp", path)
        out.append(path)
    return out


_cache = {}


def load(prec="f64"):
    if prec in ("fp32", "f32"):
        prec = "f32"
    elif prec in ("fp64", "f64"):
        prec = "f64"
    if prec in _cache:
        return _cache[prec]
    build()
    lib = ctypes.CDLL(_lib_path(prec))
    fp = ctypes.c_void_p
    lib.nutsref_run.restype = ctypes.c_int
    lib.nutsref_run.argtypes = [ctypes.c_int, fp, fp, fp, ctypes.c_int64, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_uint64, ctypes.c_int, ctypes.c_int, fp, fp, fp, fp, fp, fp,
                                ctypes.c_double]
    mp = ctypes.POINTER(NutsrefModel)
    lib.nutsref_latent_dim.restype = ctypes.c_int
    lib.nutsref_latent_dim.argtypes = [mp, ctypes.c_int]
    lib.nutsref_potential.restype = ctypes.c_double
    lib.nutsref_potential.argtypes = [mp, ctypes.c_int, fp, fp]
    lib.nutsref_transitions.restype = ctypes.c_int
    lib.nutsref_transitions.argtypes = [mp, ctypes.c_int, fp, fp, ctypes.c_int, fp, fp, fp, fp, ctypes.c_uint64,
                                        ctypes.c_int, ctypes.c_int, fp, fp, fp, fp, fp]
    lib.nutsref_run_model.restype = ctypes.c_int
    lib.nutsref_run_model.argtypes = [mp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_uint64, ctypes.c_int, ctypes.c_int, fp, fp, fp, fp, fp, fp, fp, fp,
                                      fp, ctypes.c_double]
    _cache[prec] = lib
    return lib


class NutsrefModel(ctypes.Structure):
    """nutsref_model of nuts_ref.c (the registry model, as gbn_model_desc)."""

    _fields_ = [("family", ctypes.c_int32), ("num_models", ctypes.c_int32), ("chains_per_model", ctypes.c_int32),
                ("P", ctypes.c_int32), ("N", ctypes.c_int64), ("X", ctypes.c_void_p), ("y", ctypes.c_void_p),
                ("sigma", ctypes.c_void_p), ("offsets", ctypes.c_void_p), ("hyper", ctypes.c_double * 4),
                ("row_threads", ctypes.c_int32), ("target_accept", ctypes.c_double)]


class Model:
    """Keeps the arrays of a NutsrefModel alive.  kind: hier_nc, logreg, horseshoe,
    horseshoe_nc, sv, sv_nc (as oracle.potentials_ref.FAMILIES)."""

    def __init__(self, kind, X=None, y=None, sigma=None, offsets=None, chains_per_model=1, hyper=None,
                 row_threads=0, target_accept=0.8):
        fam = {"hier_nc": 1, "logreg": 2, "horseshoe": 3, "horseshoe_nc": 3, "sv": 4, "sv_nc": 4}[kind]
        self.kind = kind
        self.X = None if X is None else np.ascontiguousarray(X, np.float32)
        self.y = np.ascontiguousarray(y, np.float32)
        self.sigma = None if sigma is None else np.ascontiguousarray(sigma, np.float32)
        self.offsets = None if offsets is None else np.ascontiguousarray(offsets, np.int32)
        h = [0.0] * 4
        if kind == "hier_nc":
            h[:2] = [5.0, 5.0]
        elif kind == "logreg":
            h[0] = 1.0
        elif kind == "horseshoe_nc":
            h[0] = 1.0
        elif kind in ("sv", "sv_nc"):
            h[:3] = [10.0, 0.1, 1.0 if kind == "sv_nc" else 0.0]
        if hyper is not None:
            h[:len(hyper)] = list(hyper)
        s = NutsrefModel()
        s.family = fam
        s.num_models = 1 if self.offsets is None else len(self.offsets) - 1
        s.chains_per_model = chains_per_model
        s.P = 0 if self.X is None else self.X.shape[1]
        s.N = len(self.y) if fam != 1 or self.offsets is None else int(self.offsets[-1])
        if fam == 1 and self.offsets is None:
            s.N = len(self.y)
        s.X = _p(self.X)
        s.y = _p(self.y)
        s.sigma = _p(self.sigma)
        s.offsets = _p(self.offsets)
        s.hyper = (ctypes.c_double * 4)(*h)
        s.row_threads = int(row_threads)
        s.target_accept = float(target_accept)
        self.struct = s

    def ref(self):
        return ctypes.byref(self.struct)


def model_from_registry(model, chains_per_model=1):
    """The C restatement's copy of a numpyro_gb300 registry model, read from its public
    attributes (datasets / X, y / returns and the family's options)."""
    kind = type(model).__name__
    if kind == "HierarchicalNormal":
        y = np.concatenate([a for a, _ in model.datasets])
        s = np.concatenate([b for _, b in model.datasets])
        off = np.zeros(len(model.datasets) + 1, np.int32)
        off[1:] = np.cumsum([len(a) for a, _ in model.datasets])
        return Model("hier_nc", y=y, sigma=s, offsets=off, chains_per_model=chains_per_model,
                     hyper=(model.mu_scale, model.tau_scale))
    if kind == "LogisticRegression":
        return Model("logreg", X=model.X, y=model.y, hyper=(model.prior_scale,))
    if kind == "HorseshoeRegression":
        return Model("horseshoe_nc" if model.noncentered else "horseshoe", X=model.X, y=model.y)
    if kind == "StochasticVolatility":
        return Model("sv_nc" if model.noncentered else "sv", y=model.returns,
                     hyper=(model.s_rate, model.nu_rate, 1.0 if model.noncentered else 0.0))
    raise TypeError("no C restatement of %s" % kind)


def potential(lib, model, z, model_index=0):
    """(U, dU/dz) of one point, from the C restatement (FP64 with the f64 build)."""
    z = np.ascontiguousarray(z, np.float64)
    g = np.zeros_like(z)
    pe = lib.nutsref_potential(model.ref(), model_index, _p(z), _p(g))
    return pe, g


def transitions(lib, model, z0, step, inv, msq, chain_ids, iters, seed, max_tree_depth=10, threads=0):
    """One NUTS transition per row of z0 (see nutsref_transitions in nuts_ref.c)."""
    z0 = np.ascontiguousarray(z0, np.float32)
    C, ld = z0.shape
    step = np.ascontiguousarray(np.broadcast_to(step, (C,)), np.float32)
    inv = np.ascontiguousarray(np.broadcast_to(inv, (C, ld)), np.float32)
    msq = np.ascontiguousarray(np.broadcast_to(msq, (C, ld)), np.float32)
    ids = np.ascontiguousarray(np.broadcast_to(chain_ids, (C,)), np.uint32)
    its = np.ascontiguousarray(np.broadcast_to(iters, (C,)), np.uint32)
    z = np.zeros((C, ld), np.float32)
    ns = np.zeros(C, np.int32)
    ap = np.zeros(C, np.float64)
    dv = np.zeros(C, np.uint8)
    pe = np.zeros(C, np.float64)
    lib.nutsref_transitions(model.ref(), C, _p(ids), _p(its), ld, _p(z0), _p(step), _p(inv), _p(msq), int(seed),
                            max_tree_depth, threads, _p(z), _p(ns), _p(ap), _p(dv), _p(pe))
    return {"z": z, "num_steps": ns, "accept_prob": ap, "diverging": dv.astype(bool), "potential_energy": pe}


def run_model(lib, model, ld, chains, num_warmup, num_samples, seed=0, first_chain=0, max_tree_depth=10, threads=0,
              init=None, warmup_budget_s=0.0):
    """Warmup (Stan windows, diagonal mass) + sampling of `chains` chains of `model`."""
    S = max(num_samples, 0)
    samples = np.zeros((chains, S, ld), np.float32)
    nsteps = np.zeros((chains, S), np.int32)
    div = np.zeros((chains, S), np.uint8)
    astep = np.zeros(chains, np.float32)
    ainv = np.zeros((chains, ld), np.float32)
    timing = np.zeros(5, np.float64)
    iz = istep = iinv = None
    if init is not None:
        iz = np.ascontiguousarray(init[0], np.float32)
        istep = np.ascontiguousarray(init[1], np.float32)
        iinv = np.ascontiguousarray(init[2], np.float32)
    lib.nutsref_run_model(model.ref(), ld, chains, first_chain, num_warmup, num_samples, int(seed), max_tree_depth,
                          threads, _p(iz), _p(istep), _p(iinv), _p(samples), _p(nsteps), _p(div), _p(astep),
                          _p(ainv), _p(timing), float(warmup_budget_s))
    return {"samples": samples, "num_steps": nsteps, "diverging": div.astype(bool), "step_size": astep,
            "inverse_mass_matrix": ainv, "warmup_s": timing[0], "sampling_s": timing[1],
            "warmup_grad_evals": timing[2], "sampling_grad_evals": timing[3], "threads": int(timing[4]),
            "chains": chains}


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run(lib, family, X=None, y=None, sigma=None, N=0, D=0, hyper=(0.0, 0.0), chains=1, first_chain=0,
        num_warmup=0, num_samples=0, seed=0, max_tree_depth=10, threads=0, init=None, warmup_budget_s=0.0):
    """init: optional (z [chains, D], step [chains], inv_mass [chains, D]) -> no adaptation."""
    samples = np.zeros((chains, max(num_samples, 0), D), np.float32)
    nsteps = np.zeros((chains, max(num_samples, 0)), np.int32)
    timing = np.zeros(5, np.float64)
    iz = istep = iinv = None
    if init is not None:
        iz = np.ascontiguousarray(init[0], np.float32)
        istep = np.ascontiguousarray(init[1], np.float32)
        iinv = np.ascontiguousarray(init[2], np.float32)
    keep = [np.ascontiguousarray(a, np.float32) if a is not None else None for a in (X, y, sigma)]
    lib.nutsref_run(family, _p(keep[0]), _p(keep[1]), _p(keep[2]), int(N), int(D), float(hyper[0]),
                    float(hyper[1]), chains, first_chain, num_warmup, num_samples, int(seed), max_tree_depth,
                    threads, _p(iz), _p(istep), _p(iinv), _p(samples), _p(nsteps), _p(timing),
                    float(warmup_budget_s))
    return {"samples": samples, "num_steps": nsteps, "warmup_s": timing[0], "sampling_s": timing[1],
            "warmup_grad_evals": timing[2], "sampling_grad_evals": timing[3], "threads": int(timing[4]),
            "chains": chains}


def run_logreg(lib, X, y, chains, num_warmup, num_samples, seed=0, threads=0, init=None, first_chain=0,
               warmup_budget_s=0.0):
    X = np.ascontiguousarray(X, np.float32)
    return run(lib, 2, X=X, y=y, N=X.shape[0], D=X.shape[1], hyper=(1.0, 0.0), chains=chains,
               first_chain=first_chain, num_warmup=num_warmup, num_samples=num_samples, seed=seed,
               threads=threads, init=init, warmup_budget_s=warmup_budget_s)


def run_hier(lib, y, sigma, chains, num_warmup, num_samples, seed=0, threads=0):
    return run(lib, 1, y=y, sigma=sigma, N=len(y), D=len(y) + 2, hyper=(5.0, 5.0), chains=chains,
               num_warmup=num_warmup, num_samples=num_samples, seed=seed, threads=threads)
