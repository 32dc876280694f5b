"""ctypes binding of the engine's C ABI (include/ekgsim.h).

The shared library is loaded from the package directory.  There is no fallback: when the
library is missing, or the process has no CUDA device, calls fail with ``EkgError``.
"""
from __future__ import annotations

import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libekgsim_gb300.so")

EKG_OK = 0
ERRORS = {
    -1: "EKG_ERR_BAD_INPUT", -2: "EKG_ERR_OUT_OF_MEMORY", -3: "EKG_ERR_CA_NOT_CONVERGED", -4: "EKG_ERR_DEVICE",
    -5: "EKG_ERR_TIMEOUT", -6: "EKG_ERR_NO_START", -7: "EKG_ERR_TRANSFER", -8: "EKG_ERR_IO",
    -9: "EKG_ERR_NOT_FOUND", -10: "EKG_ERR_BUSY",
}
NHOOD = {"3D4": 0, "3D8": 1, "cube": 1, "2D4": 2, "2D8": 3}

c_int32, c_int64, c_uint32, c_uint64, c_double = (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32,
                                                   ctypes.c_uint64, ctypes.c_double)
P = ctypes.POINTER


class EkgError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERRORS.get(code, code)}: {message}")
        self.code = code
        self.message = message


class HeartDesc(ctypes.Structure):
    _fields_ = [("nz", c_int32), ("ny", c_int32), ("nx", c_int32), ("layers", P(c_int32)),
                ("n_transfer", c_int32), ("transfer", P(c_double)), ("n_leads", c_int32),
                ("leads_zyx", P(c_double)), ("nhood", c_int32), ("start", c_double), ("length", c_double),
                ("dt", c_double), ("activation_in", P(c_double))]


class HeartInfo(ctypes.Structure):
    _fields_ = [("n_cells", c_int64), ("n_voxels", c_int64), ("n_aps", c_int64), ("n_layers", c_int32),
                ("n_leads", c_int32), ("steps", c_int32), ("ca_rounds", c_int32), ("device_bytes", c_int64),
                ("ca_ms", c_double), ("setup_ms", c_double), ("ca_buckets", c_int32)]


class EvalConfig(ctypes.Structure):
    _fields_ = [("interpolation", c_int32), ("mid_position", c_double), ("n_base_aps", c_int32),
                ("base_aps", P(c_double)), ("k_min", P(c_double)), ("k_max", P(c_double)),
                ("free_k_mask", c_uint32), ("optimize_points", c_int32), ("criteria_mode", c_int32),
                ("comparison_mode", c_int32), ("peak_is_criterion", c_int32), ("fast_is_criterion", c_int32),
                ("fast_delay", c_double), ("fast_limit", c_double), ("endo_epi_delay", c_double),
                ("n_targets", c_int32), ("target_len", P(c_int64)), ("targets", P(c_double)),
                ("target_offsets", P(c_double)), ("n_disp_min", c_int32), ("disp_min", P(c_double)),
                ("n_disp_max", c_int32), ("disp_max", P(c_double))]


class ServerOpts(ctypes.Structure):
    _fields_ = [("max_batch", c_int32), ("max_wait_us", c_int32), ("hbm_reserve_bytes", c_uint64),
                ("no_ecg", c_int32)]


class RequestStats(ctypes.Structure):
    _fields_ = [("queue_ms", c_double), ("total_ms", c_double), ("batch_size", c_int32)]


# name -> (restype, argtypes); every symbol include/ekgsim.h declares
SIGNATURES = {
    "ekg_last_error": (ctypes.c_char_p, []),
    "ekg_engine_create": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_void_p)]),
    "ekg_engine_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ekg_engine_free_bytes": (ctypes.c_int, [ctypes.c_void_p, P(c_uint64)]),
    "ekg_heart_create": (ctypes.c_int, [ctypes.c_void_p, P(HeartDesc), P(ctypes.c_void_p)]),
    "ekg_heart_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ekg_heart_get_info": (ctypes.c_int, [ctypes.c_void_p, P(HeartInfo)]),
    "ekg_heart_time_axis": (ctypes.c_int, [ctypes.c_void_p, P(c_double), P(c_double), P(c_double)]),
    "ekg_heart_activation": (ctypes.c_int, [ctypes.c_void_p, P(c_double)]),
    "ekg_heart_ap_index": (ctypes.c_int, [ctypes.c_void_p, P(c_int64)]),
    "ekg_simulate": (ctypes.c_int, [ctypes.c_void_p, P(c_double), P(c_double), P(c_double)]),
    "ekg_heart_benchmark": (ctypes.c_int, [ctypes.c_void_p, c_int32, P(c_double), P(c_double), c_int32, c_int32,
                                           P(c_double), c_int32]),
    "ekg_heart_set_eval": (ctypes.c_int, [ctypes.c_void_p, P(EvalConfig)]),
    "ekg_eval_shape": (ctypes.c_int, [ctypes.c_void_p, P(c_int32), P(c_int32)]),
    "ekg_eval_gene_bounds": (ctypes.c_int, [ctypes.c_void_p, P(c_double), P(c_double)]),
    "ekg_eval": (ctypes.c_int, [ctypes.c_void_p, P(c_double), c_int32, P(c_double), P(c_double), P(c_double),
                                P(c_double), P(c_double)]),
    "ekg_eval_simulated": (ctypes.c_int, [ctypes.c_void_p, P(c_int32)]),
    # raw addresses (array.ctypes.data): the batched call is on the per-step path, where ctypes
    # pointer objects cost more than the call itself
    "ekg_eval_batch": (ctypes.c_int, [ctypes.c_void_p, c_int32, ctypes.c_void_p, c_int32, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "ekg_eval_batch_submit": (ctypes.c_int, [ctypes.c_void_p, c_int32, ctypes.c_void_p, c_int32, ctypes.c_void_p,
                                             ctypes.c_void_p, ctypes.c_void_p, P(ctypes.c_int64)]),
    "ekg_eval_batch_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "ekg_host_register": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "ekg_host_unregister": (ctypes.c_int, [ctypes.c_void_p]),
    "ekg_server_create": (ctypes.c_int, [ctypes.c_void_p, P(ServerOpts), P(ctypes.c_void_p)]),
    "ekg_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ekg_server_add_heart": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, P(c_int32)]),
    "ekg_server_submit": (ctypes.c_int, [ctypes.c_void_p, c_int32, P(c_double), c_int32, P(c_uint64)]),
    "ekg_server_poll": (ctypes.c_int, [ctypes.c_void_p, c_uint64, c_int32, P(c_double), P(c_double), P(c_double),
                                       P(RequestStats)]),
    "ekg_server_submit_many": (ctypes.c_int, [ctypes.c_void_p, c_int32, P(c_int32), P(c_double), c_int32,
                                              P(c_uint64)]),
    "ekg_server_poll_many": (ctypes.c_int, [ctypes.c_void_p, c_int32, P(c_uint64), c_int32, c_int32, P(c_double),
                                            P(c_double), P(c_int32), P(RequestStats)]),
    "ekg_heart_tune": (ctypes.c_int, [ctypes.c_void_p, c_int32, P(c_double), P(c_double), c_int32, P(c_double),
                                      c_int32]),
    "ekg_tune_candidates": (ctypes.c_int, [c_int32, c_int32, c_int32, P(c_int32), c_int32, P(c_int32)]),
    "ekg_tune_cache_put": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, P(c_int32), c_double]),
    "ekg_tune_cache_get": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, P(c_int32), P(c_double)]),
    "ekg_selftest_bounded_wait": (ctypes.c_int, [c_int32, ctypes.c_uint32]),
    "ekg_server_set_free_bytes_provider": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ekg_activation_noalloc": (ctypes.c_int, [c_int32, c_int32, c_int32, ctypes.c_void_p, c_int32, P(c_double),
                                              ctypes.c_void_p, P(c_int32)]),
    "ekg_heart_from_ini": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, P(ctypes.c_void_p)]),
    "ekg_ap_value": (c_double, [P(c_double), c_double, c_double]),
    "ekg_heart_cell_ap": (ctypes.c_int, [ctypes.c_void_p, c_int64, P(c_int32), P(c_double)]),
    "ekg_move_leads": (ctypes.c_int, [c_int32, P(c_double), P(c_double), P(c_double)]),
    "ekg_layer_aps": (ctypes.c_int, [P(EvalConfig), c_int32, P(c_double), P(c_double), P(c_double)]),
}

_lib = None


def load():
    """Load the engine library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _b
        _b.build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != EKG_OK:
        msg = load().ekg_last_error()
        raise EkgError(code, msg.decode() if msg else "")


def dptr(a):
    return None if a is None else a.ctypes.data_as(P(c_double))


def i32ptr(a):
    return a.ctypes.data_as(P(c_int32))


def i64ptr(a):
    return a.ctypes.data_as(P(c_int64))
