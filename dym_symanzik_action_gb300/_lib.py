"""ctypes binding of libdymgpu.so (include/dymgpu.h).

The shared library is built in-tree by dym_symanzik_action_gb300.build; there
is no pure-Python or CPU fallback: if the library is missing, importing the
engine fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "lib", "libdymgpu.so")

DYM_OK = 0
ERRORS = {-1: "DYM_EINVAL", -2: "DYM_EIO", -3: "DYM_EFORMAT", -4: "DYM_ENOMEM", -5: "DYM_ECUDA",
          -6: "DYM_ENOTSUP", -7: "DYM_ETIMEDOUT", -8: "DYM_ERANGE"}
START = {"hot": 0, "cold": 1}
POOL = {"nearest": 0, "all": 1}
PRECISION = {"fp64": 0, "mixed": 1, "shared": 2}


class DymError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class GroupInfo(C.Structure):
    _fields_ = [("order", C.c_uint32), ("identity", C.c_uint32), ("pool_nearest", C.c_uint32),
                ("min_retr", C.c_double), ("nn_retr", C.c_double), ("n_classes", C.c_int32),
                ("classes_exact", C.c_int32), ("fast_path", C.c_int32), ("class_spread", C.c_double)]


class ChainParams(C.Structure):
    _fields_ = [("D", C.c_int32), ("Nt", C.c_int32), ("Nx", C.c_int32), ("beta0", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double), ("seed", C.c_uint64), ("start", C.c_int32),
                ("pool", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32)]


class CheckpointInfo(C.Structure):
    _fields_ = [("D", C.c_int32), ("Nt", C.c_int32), ("Nx", C.c_int32), ("order", C.c_uint32), ("pool", C.c_int32),
                ("table_hash", C.c_uint64), ("seed", C.c_uint64), ("sweep", C.c_uint32), ("beta0", C.c_double),
                ("beta1", C.c_double), ("beta2", C.c_double)]


class Stats(C.Structure):
    _fields_ = [("hits", C.c_uint64), ("accepts", C.c_uint64), ("rechecks", C.c_uint64),
                ("max_ds_err", C.c_double), ("sweep", C.c_uint32), ("launches", C.c_uint32),
                ("device_ms", C.c_float), ("kernel", C.c_int32)]


class MeasOpts(C.Structure):
    _fields_ = [("wl_nx", C.c_int32), ("wl_nt", C.c_int32)]


class Obs(C.Structure):
    _fields_ = [("poly_re", C.c_double), ("poly_im", C.c_double), ("plaq", C.c_double), ("rect", C.c_double),
                ("wl_nx", C.c_int32), ("wl_nt", C.c_int32)]


class LlrReq(C.Structure):
    _fields_ = [("axis", C.c_int32), ("bg", C.c_double), ("ewin", C.c_double), ("hw", C.c_double),
                ("a0", C.c_double), ("K", C.c_int32), ("NRM", C.c_int32), ("nhit", C.c_int32),
                ("drive_cap", C.c_int32)]


class LlrResult(C.Structure):
    _fields_ = [("a", C.c_double), ("S1", C.c_double), ("S2", C.c_double), ("status", C.c_int32),
                ("drive_sweeps", C.c_int32), ("sweeps", C.c_int32), ("hits", C.c_uint64), ("accepts", C.c_uint64),
                ("phase_accepts", C.c_uint64), ("phase_rejects", C.c_uint64)]


class Llr2dReq(C.Structure):
    _fields_ = [("E1", C.c_double), ("hw1", C.c_double), ("E2", C.c_double), ("hw2", C.c_double),
                ("a1", C.c_double), ("a2", C.c_double), ("K", C.c_int32), ("NRM", C.c_int32), ("nhit", C.c_int32),
                ("drive_cap", C.c_int32)]


class Llr2dResult(C.Structure):
    _fields_ = [("a1", C.c_double), ("a2", C.c_double), ("S1", C.c_double), ("S2", C.c_double),
                ("status", C.c_int32), ("drive_sweeps", C.c_int32), ("sweeps", C.c_int32), ("hits", C.c_uint64),
                ("accepts", C.c_uint64), ("phase_accepts", C.c_uint64), ("phase_rejects", C.c_uint64)]


class BatchTuning(C.Structure):
    _fields_ = [("tile", C.c_int32), ("threads", C.c_int32), ("grid_per_sm", C.c_int32), ("use_graph", C.c_int32),
                ("hit_unroll", C.c_int32)]


SERVE_MAX_NRM = 64


class ServerParams(C.Structure):
    _fields_ = [("max_chains", C.c_int32), ("hbm_budget", C.c_uint64), ("nhit", C.c_int32), ("device", C.c_int32),
                ("max_links", C.c_uint64)]


class LlrRequest(C.Structure):
    _fields_ = [("id", C.c_uint64), ("D", C.c_int32), ("Nt", C.c_int32), ("Nx", C.c_int32), ("start", C.c_int32),
                ("seed", C.c_uint64), ("axis", C.c_int32), ("bg", C.c_double), ("ewin", C.c_double),
                ("hw", C.c_double), ("a0", C.c_double), ("K", C.c_int32), ("NRM", C.c_int32),
                ("drive_cap", C.c_int32)]


class LlrResponse(C.Structure):
    _fields_ = [("id", C.c_uint64), ("a", C.c_double), ("S1", C.c_double), ("S2", C.c_double),
                ("status", C.c_int32), ("sweeps", C.c_int32), ("drive_sweeps", C.c_int32), ("NRM", C.c_int32),
                ("hits", C.c_uint64), ("accepts", C.c_uint64), ("a_hist", C.c_double * SERVE_MAX_NRM)]


LLR_STATUS = {0: "drive", 1: "settle", 2: "rm", 3: "done", 4: "unreached", 5: "cancelled", 6: "rejected"}

_P = C.c_void_p
_u16p = C.POINTER(C.c_uint16)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_f64p = C.POINTER(C.c_double)

# name -> (restype, argtypes); every entry point declared in include/dymgpu.h
PROTOTYPES = {
    "dym_last_error": (C.c_char_p, []),
    "dym_version": (C.c_char_p, []),
    "dym_group_load": (C.c_int, [C.c_char_p, C.POINTER(_P)]),
    "dym_group_free": (C.c_int, [_P]),
    "dym_group_get_info": (C.c_int, [_P, C.POINTER(GroupInfo)]),
    "dym_group_get_tables": (C.c_int, [_P, _i32p, _i32p, _f64p, _f64p, _i32p]),
    "dym_chain_create": (C.c_int, [_P, C.POINTER(ChainParams), C.POINTER(_P)]),
    "dym_chain_free": (C.c_int, [_P]),
    "dym_chain_set_beta": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    "dym_chain_set_l2_window": (C.c_int, [_P, C.c_int32]),
    "dym_chain_checkpoint_save": (C.c_int, [_P, C.c_char_p]),
    "dym_chain_checkpoint_load": (C.c_int, [_P, C.c_char_p]),
    "dym_checkpoint_read_info": (C.c_int, [C.c_char_p, C.POINTER(CheckpointInfo)]),
    "dym_group_table_hash": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "dym_sweep": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(Stats)]),
    "dym_measure": (C.c_int, [_P, C.POINTER(MeasOpts), C.POINTER(Obs), _f64p]),
    "dym_measure_noalloc": (C.c_int, [_P, C.POINTER(MeasOpts), C.POINTER(Obs), _f64p]),
    "dym_links_get": (C.c_int, [_P, _u16p]),
    "dym_links_set": (C.c_int, [_P, _u16p]),
    "dym_sweep_host": (C.c_int, [_P, _u16p, _u16p, C.c_int32, C.c_int32, C.POINTER(Stats)]),
    "dym_sweep_refarray": (C.c_int, [_P, _i32p, C.c_int32, C.c_int32, C.POINTER(Stats)]),
    "dym_chain_get_schedule": (C.c_int, [_P, _u32p, _i32p, _i32p, _u32p, _u32p]),
    "dym_chain_staples": (C.c_int, [_P, C.c_int32, _u32p, C.c_int32, _u16p]),
    "dym_schedule_check": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _i32p, _u64p]),
    "dym_schedule_get": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _u32p, _i32p, _i32p, _u32p, _u32p]),
    "dym_batch_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "dym_batch_add": (C.c_int, [_P, _P]),
    "dym_batch_size": (C.c_int, [_P, _i32p, _u64p, _i32p]),
    "dym_batch_set_tuning": (C.c_int, [_P, C.POINTER(BatchTuning)]),
    "dym_batch_get_tuning": (C.c_int, [_P, C.POINTER(BatchTuning)]),
    "dym_batch_sweep": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(Stats)]),
    "dym_batch_chain_counters": (C.c_int, [_P, C.c_int32, _u64p, _u64p]),
    "dym_batch_autotune": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(BatchTuning)]),
    "dym_batch_free": (C.c_int, [_P]),
    "dym_server_create": (C.c_int, [_P, C.POINTER(ServerParams), C.POINTER(_P)]),
    "dym_server_submit": (C.c_int, [_P, C.POINTER(LlrRequest)]),
    "dym_server_cancel": (C.c_int, [_P, C.c_uint64]),
    "dym_server_step": (C.c_int, [_P, C.c_int32]),
    "dym_server_poll": (C.c_int, [_P, C.POINTER(LlrResponse), C.c_int32, _i32p]),
    "dym_server_status": (C.c_int, [_P, _i32p, _i32p, _u64p, _u64p]),
    "dym_server_free": (C.c_int, [_P]),
    "dym_llr_energy": (C.c_int, [_P, _f64p, _f64p]),
    "dym_llr_run": (C.c_int, [_P, C.POINTER(LlrReq), C.POINTER(LlrResult), _f64p]),
    "dym_llr2d_run": (C.c_int, [_P, C.POINTER(Llr2dReq), C.POINTER(Llr2dResult), _f64p]),
    "dym_probe_l2_gather": (C.c_int, [C.c_int32, C.c_uint32, _f64p]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libdymgpu.so not built ({LIB_PATH}); run "
                               "`python -m dym_symanzik_action_gb300.build` (needs nvcc)")
        l = C.CDLL(LIB_PATH)
        for name, (res, args) in PROTOTYPES.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(rc: int) -> None:
    if rc != DYM_OK:
        raise DymError(rc, lib().dym_last_error().decode(errors="replace"))


def ptr(arr, ctype):
    """ctypes pointer to a contiguous numpy array (or None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(ctype))
