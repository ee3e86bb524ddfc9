"""numpyro_gb300 -- a GB300-native (sm_103a) engine for numpyro's NUTS/HMC hot path.

Drop-in for the vectorized-chain NUTS/HMC transition of numpyro: ``NUTS`` and
``HMC`` are MCMCKernels with numpyro's constructor arguments and HMCState
fields, driven by ``MCMC(..., chain_method="vectorized")``.  The transition
(leapfrog, iterative tree building, U-turn/divergence checks, multinomial
sampling, warmup adaptation) and the model potentials with their hand-written
adjoints run in CUDA kernels of ``libgbnuts.so`` behind a C ABI
(include/gbnuts.h).  There is no CPU fallback.
"""
from . import datasets, diagnostics, models
from .hmc import HMC, NUTS, HMCAdaptState, HMCState, hmc, init_to_uniform
from .mcmc import MCMC, MCMCKernel
from .util import ModelInfo, ParamInfo, fori_collect, initialize_model

__all__ = ["HMC", "NUTS", "MCMC", "MCMCKernel", "HMCState", "HMCAdaptState", "hmc", "fori_collect",
           "initialize_model", "ModelInfo", "ParamInfo", "init_to_uniform", "models", "datasets", "diagnostics"]
__version__ = "0.1.0"
