"""ctypes binding of libmhdgb.so (the C ABI in include/mhdgb.h).

There is no fallback: if the shared library has not been built, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB
_lib = None

MHDGB_FP64, MHDGB_FP64_EXACT, MHDGB_MIXED = 0, 1, 2
PRECISIONS = {"fp64": MHDGB_FP64, "fp64_exact": MHDGB_FP64_EXACT, "mixed": MHDGB_MIXED}
RIEMANN = {"hlld": 0, "hlle": 1, "hllc": 2}
BC_EXCHANGE = 4  # a face shared with another block of a decomposed grid
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "non-finite value", -4: "non-positive rho/p",
          -5: "device wait timed out", -6: "call out of order", -7: "device allocation failed",
          -8: "grid too large for the fixed scratch", -9: "file output failed"}

# every symbol include/mhdgb.h declares, with (restype, argtypes)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("x1min", C.c_double), ("x1max", C.c_double), ("x2min", C.c_double), ("x2max", C.c_double),
                ("x3min", C.c_double), ("x3max", C.c_double), ("bc", C.c_int * 6), ("gam", C.c_double),
                ("cfl", C.c_double), ("precision", C.c_int), ("spacing_quirk", C.c_int), ("device", C.c_int)]


class Report(C.Structure):
    _fields_ = [("step", C.c_longlong), ("time", C.c_double), ("dt", C.c_double), ("chg", C.c_double),
                ("next_dt", C.c_double), ("next_chg", C.c_double), ("done", C.c_int), ("status", C.c_uint)]


SIGNATURES = {
    "mhdgb_config_default": (C.c_int, [C.POINTER(Config)]),
    "mhdgb_create": (C.c_int, [C.POINTER(Config), C.POINTER(_vp)]),
    "mhdgb_destroy": (C.c_int, [_vp]),
    "mhdgb_last_error": (C.c_char_p, [_vp]),
    "mhdgb_status_string": (C.c_char_p, [C.c_int]),
    "mhdgb_extents": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mhdgb_device_bytes": (C.c_size_t, [_vp]),
    "mhdgb_set_physics": (C.c_int, [_vp, C.c_double, C.c_double, C.POINTER(C.c_int)]),
    "mhdgb_set_riemann": (C.c_int, [_vp, C.c_int]),
    "mhdgb_get_riemann": (C.c_int, [_vp]),
    "mhdgb_get_grid": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mhdgb_set_grid": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mhdgb_upload_cons": (C.c_int, [_vp, _dp]),
    "mhdgb_upload_prim": (C.c_int, [_vp, _dp]),
    "mhdgb_download_cons": (C.c_int, [_vp, _dp]),
    "mhdgb_download_prim": (C.c_int, [_vp, _dp]),
    "mhdgb_download_flux": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_upload_cons_field": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_download_cons_field": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_upload_prim_field": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_download_prim_field": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_control_timestep": (C.c_int, [_vp, _dp]),
    "mhdgb_set_boundary": (C.c_int, [_vp]),
    "mhdgb_output_begin": (C.c_int, [_vp, C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_int]),
    "mhdgb_output_end": (C.c_int, [_vp]),
    "mhdgb_checkpoint_save": (C.c_int, [_vp, C.c_char_p]),
    "mhdgb_checkpoint_load": (C.c_int, [_vp, C.c_char_p]),
    "mhdgb_output": (C.c_int, [_vp, C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_int]),
    "mhdgb_fill_ghosts_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), _vp]),
    "mhdgb_evaluate_ch": (C.c_int, [_vp, _dp]),
    "mhdgb_flux": (C.c_int, [_vp, C.c_int]),
    "mhdgb_update_conserv": (C.c_int, [_vp]),
    "mhdgb_damp_psi": (C.c_int, [_vp]),
    "mhdgb_update_prim": (C.c_int, [_vp]),
    "mhdgb_set_dt": (C.c_int, [_vp, C.c_double]),
    "mhdgb_set_chg": (C.c_int, [_vp, C.c_double]),
    "mhdgb_prepare": (C.c_int, [_vp]),
    "mhdgb_step": (C.c_int, [_vp, C.c_int]),
    "mhdgb_set_stop": (C.c_int, [_vp, C.c_double, C.c_longlong]),
    "mhdgb_run_until": (C.c_int, [_vp, C.c_double, C.c_longlong, C.POINTER(Report)]),
    "mhdgb_sync": (C.c_int, [_vp, C.POINTER(Report)]),
    "mhdgb_reset_clock": (C.c_int, [_vp]),
    "mhdgb_step_host": (C.c_int, [_vp, _dp, _dp, C.c_int, _dp, _dp]),
    "mhdgb_time_steps": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_selftest_fused_abort": (C.c_int, [C.c_int, C.c_int, _dp, C.POINTER(C.c_uint), C.POINTER(C.c_int)]),
    "mhdgb_variant_count": (C.c_int, [_vp]),
    "mhdgb_variant_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
    "mhdgb_variant_name": (C.c_char_p, [_vp, C.c_int]),
    "mhdgb_work_layout": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    "mhdgb_select_variant": (C.c_int, [_vp, C.c_int]),
    "mhdgb_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "mhdgb_plan_zchunks": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                     C.c_int]),
    "mhdgb_measure_fp64_rate": (C.c_int, [C.c_int, _dp]),
    "mhdgb_selftest_division": (C.c_int, [C.c_int, C.c_int, C.c_ulonglong, _dp]),
    "mhdgb_selftest_wait_timeout": (C.c_int, [C.c_int, _dp, C.POINTER(C.c_uint)]),
    "mhdgb_diag": (C.c_int, [_vp, _dp]),
    "mhdgb_init_kh": (C.c_int, [_vp, C.c_ulonglong, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double]),
    "mhdgb_init_kh_block": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_ulonglong, C.c_double,
                                      C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]),
    "mhdgb_ensemble_create": (C.c_int, [C.c_int, C.POINTER(Config), C.POINTER(_vp)]),
    "mhdgb_ensemble_destroy": (C.c_int, [_vp]),
    "mhdgb_ensemble_last_error": (C.c_char_p, [_vp]),
    "mhdgb_ensemble_size": (C.c_int, [_vp]),
    "mhdgb_ensemble_member": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "mhdgb_ensemble_cells": (C.c_longlong, [_vp]),
    "mhdgb_ensemble_prepare": (C.c_int, [_vp]),
    "mhdgb_ensemble_step": (C.c_int, [_vp, C.c_int]),
    "mhdgb_ensemble_sync": (C.c_int, [_vp, C.POINTER(Report)]),
    "mhdgb_ensemble_set_stop": (C.c_int, [_vp, C.c_double, C.c_longlong]),
    "mhdgb_ensemble_time_steps": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_ensemble_select_variant": (C.c_int, [_vp, C.c_int]),
    "mhdgb_ensemble_variant": (C.c_int, [_vp]),
    "mhdgb_ensemble_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "mhdgb_halo_bytes": (C.c_size_t, [_vp, C.c_int]),
    "mhdgb_halo_pack": (C.c_int, [_vp, C.c_int, _vp]),
    "mhdgb_halo_unpack": (C.c_int, [_vp, C.c_int, _vp]),
    "mhdgb_get_reduction": (C.c_int, [_vp, _dp, _dp]),
    "mhdgb_set_reduction": (C.c_int, [_vp, C.c_double, C.c_double]),
    "mhdgb_domain_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_int),
                                      C.POINTER(_vp)]),
    "mhdgb_domain_destroy": (C.c_int, [_vp]),
    "mhdgb_domain_last_error": (C.c_char_p, [_vp]),
    "mhdgb_domain_blocks": (C.c_int, [_vp]),
    "mhdgb_domain_block": (C.c_int, [_vp, C.c_int, C.POINTER(_vp), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mhdgb_domain_upload_cons": (C.c_int, [_vp, _dp]),
    "mhdgb_domain_download_cons": (C.c_int, [_vp, _dp]),
    "mhdgb_domain_init_kh": (C.c_int, [_vp, C.c_ulonglong, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_double]),
    "mhdgb_domain_prepare": (C.c_int, [_vp]),
    "mhdgb_domain_step": (C.c_int, [_vp, C.c_int]),
    "mhdgb_domain_sync": (C.c_int, [_vp, C.POINTER(Report)]),
    "mhdgb_domain_set_stop": (C.c_int, [_vp, C.c_double, C.c_longlong]),
    "mhdgb_domain_time_steps": (C.c_int, [_vp, C.c_int, _dp]),
    "mhdgb_domain_diag": (C.c_int, [_vp, _dp]),
}


def lib(build_if_missing: bool = False):
    """Load libmhdgb.so (optionally building it first).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                                   "or python -m mhdturbulence_gb300.build (there is no CPU fallback)")
            _build.build()
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class MhdgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code
