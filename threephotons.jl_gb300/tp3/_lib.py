"""ctypes binding of libtp3.so (include/tp3.h).

The library is built in-tree (threephotons.jl_gb300/lib/libtp3.so).  Loading
fails loudly when it is missing: there is no Python or CPU fallback for any
call that computes c3 or an energy.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(_HERE)
LIB_PATH = os.path.join(PKG, "lib", "libtp3.so")

c_int, c_double, c_void_p, c_int64 = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_int64
P = ctypes.POINTER

TP3_OK = 0
TP3_ERR_ARG = 1
TP3_ERR_TABLE = 2
TP3_ERR_CUDA = 3
TP3_ERR_NO_DEVICE = 4
TP3_ERR_NO_HISTOGRAM = 5
TP3_ERR_BAD_HISTOGRAM = 6
TP3_ERR_TIMEOUT = 7
TP3_ERR_UNSUPPORTED = 8
TP3_ERR_ALLOC = 9

TP3_MODE_PLAIN_FP32 = 0
TP3_MODE_TC_BF16X3 = 1
TP3_MODE_TC_TF32X3 = 2
TP3_MODE_AUTO = -1
TP3_MOVE_REFERENCE = 0
TP3_MOVE_SHELL_SO3 = 1
TP3_MOVE_LEARNED = 2
TP3_MOVE_DRIFT = 3
TP3_ANGULAR_TILE = 0
TP3_ANGULAR_PERSISTENT = 1
TP3_HOST_INPUT_STAGED = 0
TP3_HOST_INPUT_DIRECT = 1
TP3_SH_INTENSITY = 0
TP3_SH_REFERENCE = 1

# name -> (restype, argtypes); every symbol include/tp3.h declares
SIGNATURES = {
    "tp3_status_string": (ctypes.c_char_p, [c_int]),
    "tp3_last_error": (ctypes.c_char_p, [c_void_p]),
    "tp3_version": (c_int, []),
    "tp3_wigner3j": (c_double, [c_int] * 6),
    "tp3_sphPlm": (c_double, [c_int, c_int, c_double]),
    "tp3_basis_info": (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, P(c_int64)]),
    "tp3_ctx_create": (c_int, [c_int, c_int, c_int, c_int, c_double, c_double, P(c_void_p)]),
    "tp3_ctx_destroy": (None, [c_void_p]),
    "tp3_set_stream": (c_int, [c_void_p, c_void_p]),
    "tp3_set_mode": (c_int, [c_void_p, c_int]),
    "tp3_get_mode": (c_int, [c_void_p, P(c_int)]),
    "tp3_reserve": (c_int, [c_void_p, c_int]),
    "tp3_autotune": (c_int, [c_void_p, c_int, c_void_p, P(c_int)]),
    "tp3_set_coupling": (c_int, [c_void_p, c_int]),
    "tp3_set_angular": (c_int, [c_void_p, c_int]),
    "tp3_set_host_input": (c_int, [c_void_p, c_int]),
    "tp3_retrieve_solution": (c_int, [c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int, c_int, c_double,
                                      c_double, c_void_p]),
    "tp3_fit_structures_random": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_double, c_int,
                                          c_void_p, c_void_p, c_void_p]),
    "tp3_structure_sh": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_double, c_int, c_void_p,
                                 c_void_p, c_void_p]),
    "tp3_set_histogram": (c_int, [c_void_p, c_void_p, c_int]),
    "tp3_c3": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tp3_c3_batch_device": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "tp3_triple_products": (c_int, [c_void_p, c_void_p, c_void_p]),
    "tp3_sync": (c_int, [c_void_p]),
    "tp3_energy": (c_int, [c_void_p, c_void_p, P(c_double)]),
    "tp3_energy_batch": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "tp3_energy_batch_device": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "tp3_set_histograms": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "tp3_energy_batch_ragged_device": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "tp3_ragged_limits_device": (c_int, [c_void_p, c_int, c_void_p]),
    "tp3_chains_create": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_double,
                                  ctypes.c_uint64, c_int, P(c_void_p)]),
    "tp3_chains_create_ragged": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double, c_double, c_double,
                                         ctypes.c_uint64, c_int, c_void_p, P(c_void_p)]),
    "tp3_chains_destroy": (None, [c_void_p]),
    "tp3_chains_run": (c_int, [c_void_p, c_int]),
    "tp3_chains_state": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tp3_chains_coeff": (c_int, [c_void_p, c_void_p]),
    "tp3_chains_log": (c_int, [c_void_p, c_int, c_void_p, P(c_int64)]),
    "tp3_chains_snapshot": (c_int, [c_void_p, c_void_p, ctypes.c_size_t, P(ctypes.c_size_t)]),
    "tp3_chains_restore": (c_int, [c_void_p, c_void_p, ctypes.c_size_t]),
    "tp3_chains_graph": (c_int, [c_void_p, P(c_int)]),
    "tp3_chains_set_move": (c_int, [c_void_p, c_int, c_double, c_double, c_void_p]),
    "tp3_chains_enable_move_log": (c_int, [c_void_p, c_int]),
    "tp3_chains_move_log_count": (c_int, [c_void_p, P(c_int64)]),
    "tp3_chains_move_log_gather": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "tp3_bayes_energy_noalloc": (c_int, [c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p]),
    "tp3_histogram_pictures": (c_int, [c_void_p, c_int, c_void_p, c_int64, c_void_p, c_double, c_int, c_int, c_int,
                                       c_void_p, c_void_p, c_void_p]),
    "tp3_sample_pictures": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_int, c_int, c_double, c_double, c_double,
                                    c_int, c_double, c_double, ctypes.c_uint64, c_int, c_void_p, c_void_p]),
    "tp3_sample_pictures_ex": (c_int, [c_void_p, c_int, c_int64, c_void_p, c_int, c_int, c_double, c_double,
                                       c_double, c_int, c_int, c_double, c_int, c_double, c_double, ctypes.c_uint64,
                                       c_int, c_void_p, c_void_p]),
    "tp3_intensity_max": (c_int, [c_void_p, c_void_p, c_int, c_int, c_double, c_int, c_int, P(c_double)]),
    "tp3_wigner_D": (c_int, [c_int, c_double, c_double, c_double, c_void_p]),
    "tp3_rotate_shells_device": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "tp3_mlp_create": (c_int, [c_void_p, c_int, c_int, c_int, ctypes.c_uint64, P(c_void_p)]),
    "tp3_mlp_destroy": (None, [c_void_p]),
    "tp3_mlp_num_params": (c_int, [c_void_p, P(c_int64)]),
    "tp3_mlp_get_params": (c_int, [c_void_p, c_void_p, c_int64]),
    "tp3_mlp_set_params": (c_int, [c_void_p, c_void_p, c_int64]),
    "tp3_mlp_input_buffer": (c_int, [c_void_p, P(c_void_p), P(c_int)]),
    "tp3_mlp_forward_device": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "tp3_mlp_loss_grad": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, P(c_double),
                                  c_void_p]),
    "tp3_mlp_train_step": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, ctypes.c_float,
                                   P(c_double)]),
    "tp3_selftest_timeout": (c_int, [c_void_p, ctypes.c_longlong]),
    "tp3_profile_enable": (c_int, [c_void_p, c_int]),
    "tp3_profile_read": (c_int, [c_void_p, P(c_int64), P(c_double)]),
    "tp3_profile_read_stage": (c_int, [c_void_p, c_int, P(c_int64), P(c_double)]),
    "tp3_measure_fp32_peak": (c_int, [c_void_p, P(c_double)]),
}

_lib = None


class TP3Error(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = status
        super().__init__(f"tp3 status {status} ({status_string(status)}): {detail}")


def load() -> ctypes.CDLL:
    """Load libtp3.so (building is a separate step: build.py / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libtp3.so not built at {LIB_PATH}; run threephotons.jl_gb300/build.py")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def status_string(s: int) -> str:
    return load().tp3_status_string(s).decode()


def check(status: int, ctx=None) -> None:
    if status != TP3_OK:
        detail = load().tp3_last_error(ctx).decode(errors="replace")
        raise TP3Error(status, detail)
