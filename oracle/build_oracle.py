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
    _cache[prec] = lib
    return lib


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
