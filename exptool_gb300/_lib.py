"""ctypes binding of ``libexptool_gb300.so`` (C ABI in include/exptool_gb300.h).

Device memory and streams come from PyTorch (tensors' ``data_ptr()`` and
``torch.cuda.current_stream().cuda_stream``); every compute call goes to the
CUDA library.  There is no CPU fallback: if the library or a CUDA device is
missing, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

XT_OK = 0
XT_F64 = 0
XT_F32 = 1
XT_COORD_CART = 0
XT_COORD_SPH = 1
XT_COORD_CYL = 1
XT_SPH_ALL_EVAL_PARTICLES = 0
XT_SPH_ALL_EVAL = 1
XT_SPH_FORCE_EVAL = 2
XT_CYL_ACCUMULATED_EVAL_PARTICLES = 0
XT_CYL_FORCE_EVAL = 1
XT_CYL_ACCUMULATED_EVAL = 2
XT_PTR_DEVICE = 0
XT_PTR_PINNED = 1
XT_PTR_PAGEABLE = 2
XT_PTR_INACCESSIBLE = 3
XT_COL_F32 = 0
XT_COL_F64 = 1
XT_COL_I32 = 2
XT_COL_I64 = 3
XT_COL_F32_TO_F64 = 4

_lock = threading.Lock()
_lib = None

c_int, c_ll, c_dbl, c_vp, c_sz = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
c_dp = ctypes.POINTER(ctypes.c_double)
c_dpp = ctypes.POINTER(ctypes.c_void_p)

_SIGS = {
    "xt_abi_version": (c_int, []),
    "xt_last_error": (ctypes.c_char_p, []),
    "xt_pointer_access": (c_int, [c_vp]),
    "xt_copy_async": (c_int, [c_int, c_dpp, c_dpp, ctypes.POINTER(c_sz), c_vp]),
    "xt_stream_sync": (c_int, [c_vp]),
    "xt_sph_table_create": (c_int, [c_int, c_int, c_int, c_int, c_dbl, c_dbl, c_dbl, c_vp, c_vp, c_vp, c_vp, c_vp,
                                    ctypes.POINTER(c_vp)]),
    "xt_sph_table_destroy": (c_int, [c_vp]),
    "xt_sph_accumulate_workspace": (c_sz, [c_vp]),
    "xt_sph_accumulate": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_vp, c_vp, c_sz, c_vp]),
    "xt_sph_accumulate_noalloc": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_vp, c_vp]),
    "xt_sph_field_bytes": (c_sz, [c_vp, c_int]),
    "xt_sph_prepare": (c_int, [c_vp, c_vp, c_dbl, c_int, c_int, c_int, c_vp, c_sz, c_vp]),
    "xt_sph_eval_points": (c_int, [c_vp, c_vp, c_int, c_int, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_int, c_int,
                                   c_int, c_int, c_dpp, c_vp]),
    "xt_sph_batched_workspace": (c_sz, [c_vp, c_int, c_ll, c_int]),
    "xt_sph_accumulate_batched": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp, c_sz, c_vp]),
    "xt_sph_batched_tc_workspace": (c_sz, [c_vp, c_int, c_vp, c_int]),
    "xt_sph_accumulate_batched_tc": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_int, c_vp, c_vp,
                                             c_sz, c_vp]),
    "xt_sph_batched_tc_residency": (c_int, [c_vp, c_int, c_int, c_vp]),
    "xt_sph_batched_tc_status": (c_int, []),
    "xt_cyl_table_create": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_dbl, c_dbl, c_dbl, c_dbl, c_dbl, c_dbl,
                                    c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.POINTER(c_vp)]),
    "xt_cyl_table_destroy": (c_int, [c_vp]),
    "xt_cyl_accumulate_workspace": (c_sz, [c_vp]),
    "xt_cyl_accumulate": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "xt_cyl_field_bytes": (c_sz, [c_vp, c_int, c_int]),
    "xt_cyl_prepare": (c_int, [c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_vp, c_sz, c_vp]),
    "xt_cyl_eval_points": (c_int, [c_vp, c_vp, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_int,
                                   c_int, c_int, c_int, c_dpp, c_vp]),
    "xt_cyl_accumulate_eval_workspace": (c_sz, [c_vp, c_ll, c_int]),
    "xt_cyl_accumulate_eval": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_int, c_int, c_vp, c_vp,
                                       c_dpp, c_vp, c_sz, c_vp]),
    "xt_cyl_accumulate_sorted": (c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_vp, c_vp, c_vp, c_sz,
                                         c_vp]),
    "xt_cyl_eval_sorted": (c_int, [c_vp, c_vp, c_vp, c_vp, c_ll, c_int, c_int, c_int, c_vp, c_vp, c_dpp, c_vp, c_sz,
                                   c_vp]),
    "xt_timing_enable": (c_int, [c_int]),
    "xt_cyl_field_engine": (c_int, [c_int]),
    "xt_cyl_status": (c_int, []),
    "xt_df_eval": (c_int, [c_int, c_vp, c_vp, c_ll, c_vp]),
    "xt_cyl_active_blocks": (c_int, [c_vp, c_vp, c_ll, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "xt_timing_read": (c_int, [c_dp, c_int]),
    "xt_fields_forces": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp,
                                 c_dbl, c_ll, c_dpp, c_vp]),
    "xt_orbit_sort_workspace": (c_sz, [c_vp, c_ll]),
    "xt_orbit_sort": (c_int, [c_vp, c_vp, c_vp, c_ll, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "xt_orbit_unsort": (c_int, [c_vp, c_vp, c_ll, c_vp, c_vp]),
    "xt_leapfrog": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_int, c_int, c_int, c_int, c_dpp, c_ll, c_int, c_int,
                            c_int, c_dbl, c_dbl, c_int, c_int, c_vp, c_vp, c_vp]),
    "xt_mlp_param_size": (c_int, []),
    "xt_mlp_create": (c_int, [c_int, c_int, c_vp, ctypes.POINTER(c_vp)]),
    "xt_mlp_destroy": (c_int, [c_vp]),
    "xt_mlp_workspace": (c_sz, [c_vp, c_int]),
    "xt_mlp_get": (c_int, [c_vp, c_int, c_vp]),
    "xt_mlp_set_params": (c_int, [c_vp, c_vp, c_ll]),
    "xt_mlp_forward": (c_int, [c_vp, c_vp, c_int, c_vp, c_vp, c_sz, c_vp]),
    "xt_mlp_train_step": (c_int, [c_vp, c_vp, c_vp, c_ll, c_int, ctypes.c_float, c_int, c_vp, c_vp, c_sz, c_vp]),
    "xt_mlp_labels": (c_int, [c_vp, c_int, c_vp, c_ll, c_dbl, c_vp, c_vp, c_dbl, c_dbl, c_vp, c_vp, c_ll, c_vp]),
    "xt_learned_prep_bytes": (c_sz, [c_vp, c_int]),
    "xt_learned_prepare": (c_int, [c_vp, c_vp, c_int, c_vp, c_dbl, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "xt_learned_eval_workspace": (c_sz, [c_vp, c_ll]),
    "xt_learned_eval": (c_int, [c_vp, c_vp, c_vp, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_vp, c_int, c_vp, c_ll, c_int,
                                c_int, c_vp, c_vp, c_sz, c_vp]),
    "xt_learned_radial_pass": (c_int, [c_vp, c_vp, c_vp, c_int, c_dbl, c_dbl, c_dbl, c_vp, c_int, c_vp, c_ll, c_int,
                                       c_vp, c_vp]),
    "xt_learned_status": (c_int, []),
    "xt_orbit_spectra": (c_int, [c_int, c_ll, c_int, c_vp, c_vp, c_ll, c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp,
                                 c_vp, c_vp, c_vp, c_vp, c_vp]),
    "xt_eof_basis": (c_int, [c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_dbl,
                             c_ll, c_int, c_vp, c_vp, c_vp, c_vp, c_vp]),
    "xt_records_to_columns": (c_int, [c_vp, c_ll, c_int, c_int, c_vp, c_vp, c_dpp, c_vp]),
}

EXPORTED = tuple(_SIGS)


def library_path() -> str:
    return _build.library_path()


def load(build_if_missing: bool = True):
    """Load (building first if needed) the CUDA library and bind signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"exptool_gb300 CUDA library not built: {path}")
            path = _build.build()
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class XTError(RuntimeError):
    """A failure reported by the CUDA library."""


def check(rc: int, what: str):
    if rc != XT_OK:
        msg = load().xt_last_error()
        raise XTError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")


def ptr_array(ptrs):
    """ctypes array of device pointers (0/None -> NULL)."""
    arr = (ctypes.c_void_p * len(ptrs))(*[p if p else None for p in ptrs])
    return ctypes.cast(arr, c_dpp), arr
