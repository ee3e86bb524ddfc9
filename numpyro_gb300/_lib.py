"""ctypes binding of libgbnuts.so (declared in include/gbnuts.h).

The library is built in-tree (``numpyro_gb300/libgbnuts.so``).  There is no
fallback: if it is missing or fails to load, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbnuts.so")

GBN_OK = 0
ERRORS = {
    1: "invalid argument",
    2: "shape mismatch",
    3: "CUDA error",
    4: "device timeout",
    5: "init failed",
    6: "unsupported",
    7: "out of memory",
}

FAMILY_HIER_NC, FAMILY_LOGREG, FAMILY_HORSESHOE, FAMILY_SV = 1, 2, 3, 4
ENGINE_FUSED, ENGINE_PLAIN, ENGINE_TICKS = 0, 1, 2
ALGO_NUTS, ALGO_HMC = 0, 1
PREC_FP32, PREC_BF16X3 = 0, 1

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_uint32_p = ctypes.POINTER(ctypes.c_uint32)
c_uint8_p = ctypes.POINTER(ctypes.c_uint8)


class ModelDesc(ctypes.Structure):
    _fields_ = [
        ("family", ctypes.c_int32),
        ("num_models", ctypes.c_int32),
        ("n", ctypes.c_int64),
        ("p", ctypes.c_int32),
        ("x", c_float_p),
        ("y", c_float_p),
        ("sigma", c_float_p),
        ("offsets", c_int32_p),
        ("hyper", ctypes.c_double * 8),
    ]


class Config(ctypes.Structure):
    _fields_ = [
        ("num_chains", ctypes.c_int32),
        ("chains_per_model", ctypes.c_int32),
        ("algo", ctypes.c_int32),
        ("engine", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("max_tree_depth_warmup", ctypes.c_int32),
        ("max_tree_depth", ctypes.c_int32),
        ("adapt_step_size", ctypes.c_int32),
        ("adapt_mass_matrix", ctypes.c_int32),
        ("dense_mass", ctypes.c_int32),
        ("regularize_mass_matrix", ctypes.c_int32),
        ("find_heuristic_step_size", ctypes.c_int32),
        ("num_steps", ctypes.c_int32),
        ("target_accept_prob", ctypes.c_double),
        ("trajectory_length", ctypes.c_double),
        ("max_delta_energy", ctypes.c_double),
        ("init_step_size", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("mass_blocks", c_int32_p),
        ("first_chain", ctypes.c_int32),
    ]


STATE_FIELDS = [
    ("i", c_int32_p),
    ("z", c_float_p),
    ("z_grad", c_float_p),
    ("potential_energy", c_double_p),
    ("energy", c_double_p),
    ("num_steps", c_int32_p),
    ("accept_prob", c_float_p),
    ("mean_accept_prob", c_float_p),
    ("diverging", c_uint8_p),
    ("step_size", c_float_p),
    ("inverse_mass_matrix", c_float_p),
    ("mass_matrix_sqrt", c_float_p),
    ("mass_matrix_sqrt_inv", c_float_p),
    ("ss_state", c_double_p),
    ("mm_mean", c_double_p),
    ("mm_m2", c_double_p),
    ("mm_n", c_int32_p),
    ("window_idx", c_int32_p),
    ("rng_key", c_uint32_p),
]


class State(ctypes.Structure):
    _fields_ = STATE_FIELDS


class Collect(ctypes.Structure):
    _fields_ = [
        ("samples", c_float_p),
        ("num_steps", c_int32_p),
        ("accept_prob", c_float_p),
        ("diverging", c_uint8_p),
        ("potential_energy", c_double_p),
        ("step_size", c_float_p),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("ticks", ctypes.c_int64),
        ("grad_evals", ctypes.c_int64),
        ("potential_launches", ctypes.c_int64),
        ("device_ms", ctypes.c_double),
    ]


EXPORTS = {
    "gbn_abi_version": (ctypes.c_int, []),
    "gbn_tc_available": (ctypes.c_int, []),
    "gbn_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "gbn_create": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ModelDesc), ctypes.POINTER(Config)]),
    "gbn_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "gbn_latent_dim": (ctypes.c_int, [ctypes.c_void_p, c_int32_p]),
    "gbn_potential_and_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                              ctypes.c_void_p, ctypes.c_void_p]),
    "gbn_potential_vjp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "gbn_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.POINTER(State)]),
    "gbn_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(State)]),
    "gbn_sample_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(State)]),
    "gbn_check_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "gbn_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(State), ctypes.c_int32,
                               ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(Collect)]),
    "gbn_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "gbn_tuning": (ctypes.c_char_p, [ctypes.c_void_p]),
    "gbn_measure_sfu": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_double)]),
    "gbn_logreg_terms": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float)]),
    "gbn_time_potential": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_float)]),
    "gbn_logreg_potential_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                    ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                                    ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                                    ctypes.c_void_p]),
    "gbn_noalloc_last_error": (ctypes.c_char_p, []),
    "gbn_handle_id": (ctypes.c_int64, [ctypes.c_void_p]),
    "gbn_handle_from_id": (ctypes.c_void_p, [ctypes.c_int64]),
}
NOALLOC_MAX_POINTS = 256  # GBN_NOALLOC_MAX_POINTS in include/gbnuts.h

_lib = None


class GbnError(RuntimeError):
    pass


def load():
    """Load libgbnuts.so (raises if absent: there is no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GbnError(
            "libgbnuts.so is not built (%s); run `python -m numpyro_gb300.build` "
            "or __graft_entry__.build() first -- there is no CPU fallback." % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status, handle=None):
    if status != GBN_OK:
        lib = load()
        msg = lib.gbn_last_error(handle)
        msg = msg.decode() if msg else ""
        raise GbnError("gbnuts: %s (status %d): %s" % (ERRORS.get(status, "error"), status, msg))
