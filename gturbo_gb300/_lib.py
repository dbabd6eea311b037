"""ctypes binding of ``libgturbo_gb300.so`` (the C-ABI of ``include/gturbo.h``).

There is no fallback: if the library is missing or cannot be loaded, ``load()`` raises.
"""
from __future__ import annotations

import ctypes
import os
import re

from .params import GtInfo, GtParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libgturbo_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "gturbo.h")

GT_OK = 0
ERRORS = {1: "GT_ERR_ARG", 2: "GT_ERR_CUDA", 3: "GT_ERR_NFORC", 4: "GT_ERR_STATE",
          5: "GT_ERR_NOMEM", 6: "GT_ERR_NONFINITE"}

_lib = None


class GturboError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def header_functions() -> list[str]:
    """Names of every function declared in include/gturbo.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gt_[a-z0-9_]+)\s*\(", text)))


def load(path: str | None = None):
    """Load the CUDA library (build it first with ``gturbo_gb300.build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("GTURBO_LIB") or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"gturbo_gb300 CUDA library not built: {path} is missing "
                          "(run gturbo_gb300.build.build())")
    lib = ctypes.CDLL(path)
    lib._gt_path = path
    P = ctypes.c_void_p
    D = ctypes.c_void_p  # device pointers are passed as integers
    H = ctypes.POINTER(ctypes.c_double)
    I32P = ctypes.POINTER(ctypes.c_int32)
    sig = {
        "gt_create": ([ctypes.POINTER(GtParams), ctypes.POINTER(P)], ctypes.c_int),
        "gt_destroy": ([P], ctypes.c_int),
        "gt_set_stream": ([P, P], ctypes.c_int),
        "gt_get_info": ([P, ctypes.POINTER(GtInfo)], ctypes.c_int),
        "gt_get_forcing_modes": ([P, I32P, I32P, I32P], ctypes.c_int),
        "gt_last_error": ([P], ctypes.c_char_p),
        "gt_sync": ([P], ctypes.c_int),
        "gt_fft_dir": ([P, D], ctypes.c_int),
        "gt_fft_inv": ([P, D], ctypes.c_int),
        "gt_trunc": ([P, D], ctypes.c_int),
        "gt_dump_real4": ([P, D, D], ctypes.c_int),
        "gt_load_real4": ([P, D, D], ctypes.c_int),
        "gt_produ": ([P, D, D, D], ctypes.c_int),
        "gt_nlt": ([P, D, D, D], ctypes.c_int),
        "gt_step_rk2": ([P, D, D, D, D], ctypes.c_int),
        "gt_step_rk4": ([P, D, D, D, D, D], ctypes.c_int),
        "gt_forcing": ([P, D, I32P], ctypes.c_int),
        "gt_step_rk2_forced": ([P, D, D, D, D, I32P], ctypes.c_int),
        "gt_set_col_split": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_get_col_split": ([P, I32P], ctypes.c_int),
        "gt_set_pdl": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_get_pdl": ([P, I32P], ctypes.c_int),
        "gt_set_graphs": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_get_graphs": ([P, I32P], ctypes.c_int),
        "gt_adj_set_memory": ([P, ctypes.c_int64], ctypes.c_int),
        "gt_adj_get_memory": ([P, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "gt_step_rk4_forced": ([P, D, D, D, D, D, I32P], ctypes.c_int),
        "gt_rann": ([I32P], ctypes.c_float),
        "gt_diag": ([P, D, D, H, H, H, H, H], ctypes.c_int),
        "gt_diag_static": ([ctypes.POINTER(GtParams), D, D, D, D, D, D, D, P], ctypes.c_int),
        "gt_forcing_philox": ([P, D, ctypes.c_uint64, ctypes.c_uint64], ctypes.c_int),
        "gt_objective": ([P, D, ctypes.c_double, ctypes.c_double, H, D], ctypes.c_int),
        "gt_tlm_step_rk2": ([P, D, D, ctypes.c_double, I32P, ctypes.POINTER(P)], ctypes.c_int),
        "gt_adj_stage": ([P, D, D, ctypes.POINTER(P)], ctypes.c_int),
        "gt_adj_step_rk2": ([P, D, D, D, ctypes.c_int32, H, ctypes.POINTER(P)], ctypes.c_int),
        "gt_adj_gradient": ([P, D, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                             ctypes.c_double, H, D, H, D, H], ctypes.c_int),
        "gt_tlm_run": ([P, D, D, ctypes.c_double, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                        ctypes.c_double, H, H], ctypes.c_int),
        "gt_ens_create": ([ctypes.POINTER(GtParams), ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                           ctypes.POINTER(P)], ctypes.c_int),
        "gt_ens_destroy": ([P], ctypes.c_int),
        "gt_ens_set_stream": ([P, P], ctypes.c_int),
        "gt_ens_set_fields": ([P, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P),
                               ctypes.POINTER(P), ctypes.POINTER(P)], ctypes.c_int),
        "gt_ens_set_step": ([P, ctypes.c_uint64], ctypes.c_int),
        "gt_ens_get_step": ([P, ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
        "gt_ens_use_graph": ([P, ctypes.c_int], ctypes.c_int),
        "gt_ens_step": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_ens_set_tile": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_ens_get_tile": ([P, I32P], ctypes.c_int),
        "gt_ens_autotune": ([P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), I32P], ctypes.c_int),
        "gt_ens_last_error": ([P], ctypes.c_char_p),
        "gt_profile": ([P, ctypes.c_int], ctypes.c_int),
        "gt_profile_read": ([P, H, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "gt_variant_supported": ([ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "gt_set_variant": ([P, ctypes.c_int32], ctypes.c_int),
        "gt_get_variant": ([P, I32P], ctypes.c_int),
        "gt_autotune": ([P, ctypes.c_int32, H, I32P], ctypes.c_int),
        "gt_row_variant_supported": ([ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "gt_set_variants": ([P, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
        "gt_get_variants": ([P, I32P, I32P], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def check(lib, h, rc: int) -> None:
    if rc != GT_OK:
        msg = lib.gt_last_error(h)
        raise GturboError(rc, msg.decode() if msg else "")
