"""ctypes binding of libaxs_gb300.so (the C ABI declared in include/axs.h).

The library is loaded from the package directory and nowhere else. A missing
or unloadable library raises immediately: there is no CPU fallback for any
entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from ._build import LIB_PATH

_dbl, _i32, _i64, _u64, _ptr = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p

AXS_OK = 0
AXS_ERR_INVALID_ARGUMENT = 1
AXS_ERR_UNSUPPORTED = 2
AXS_ERR_ALIGNMENT = 3
AXS_ERR_WORKSPACE = 4
AXS_ERR_CUDA = 5
AXS_ERR_DEVICE_TIMEOUT = 6
AXS_ERR_CAPACITY = 7

AXS_DEFAULT_WAIT_POLLS = 4194304

AXS_F32, AXS_F64 = 1, 2
LEVEL_COMPENSATED_FP32 = 1  # axs_level.flags
BG_EXPANDING, BG_FLAT, BG_PRE_EVOLUTION = 0, 1, 2
MASK_NONE, MASK_A, MASK_B = 0, 1, 2
BOUNDARY_GHOSTS, BOUNDARY_PERIODIC = 0, 1


class Fab(C.Structure):
    _fields_ = [("data", _ptr), ("dtype", _i32), ("nx", _i32), ("ny", _i32), ("nz", _i32), ("ng", _i32),
                ("ncomp", _i32), ("jstride", _i64), ("kstride", _i64), ("cstride", _i64)]


class RhsCoeffs(C.Structure):
    _fields_ = [("kappa", _dbl), ("lambda_", _dbl), ("R2", _dbl)]


class BackgroundC(C.Structure):
    _fields_ = [("kind", _i32), ("has_switch", _i32), ("a_inv", _dbl), ("c0", _dbl), ("c1", _dbl),
                ("tau_switch", _dbl), ("lambda_scale", _dbl), ("m_r", _dbl), ("gamma_pre", _dbl),
                ("blend_dtau", _dbl), ("blend_tau_start", _dbl), ("blend_lambda_start", _dbl),
                ("blend_curv_start", _dbl)]


class BackgroundValues(C.Structure):
    _fields_ = [("R", _dbl), ("R_prime", _dbl), ("kappa", _dbl), ("lambda_", _dbl), ("H", _dbl), ("R2", _dbl),
                ("m_r", _dbl), ("R_prime_over_R", _dbl)]


class LevelLayout(C.Structure):
    _fields_ = [("jstride", _i64), ("kstride", _i64), ("cstride", _i64), ("x_offset", _i32), ("y_offset", _i32),
                ("state_bytes", _i64), ("work_bytes", _i64)]


class LevelC(C.Structure):
    _fields_ = [("state", _ptr), ("work", _ptr), ("dtype", _i32), ("nx", _i32), ("ny", _i32), ("nz", _i32),
                ("dx", _dbl), ("tile_config", _i32), ("flags", _i32)]


class DiagParams(C.Structure):
    _fields_ = [("dx", _dbl), ("R", _dbl), ("lambda_", _dbl), ("R_prime_over_R", _dbl), ("m_r", _dbl),
                ("masking_scheme", _i32), ("masking_threshold", _dbl), ("boundary", _i32),
                ("want_energy", _i32), ("want_plaquettes", _i32), ("want_velocity", _i32),
                ("per_cell_fp32", _i32)]


class DiagResult(C.Structure):
    _fields_ = [("energy_sums", _dbl * 14), ("vel_sum", _dbl), ("vel_count", _i64), ("n_p_plain", _i64),
                ("n_p_weighted", _i64), ("n_listed", _i64), ("n_near_tie", _i64), ("status", _i64)]


class PatchLayout(C.Structure):
    _fields_ = [("jstride", _i64), ("kstride", _i64), ("patch_elems", _i64), ("plane_elems", _i64),
                ("x_offset", _i32), ("y_offset", _i32), ("z_offset", _i32), ("state_bytes", _i64),
                ("work_bytes", _i64), ("table_bytes", _i64)]


class PatchesC(C.Structure):
    _fields_ = [("dtype", _i32), ("n", _i32), ("npatches", _i32), ("dx", _dbl), ("state", _ptr), ("work", _ptr),
                ("table", _ptr), ("state_bytes", _i64), ("work_bytes", _i64), ("table_bytes", _i64),
                ("capacity", _i32)]


PATCH_KEEP = -2


class PatchPlan(C.Structure):
    _fields_ = [("items_a", _i64), ("items_b", _i64), ("grid_a", _i32), ("grid_b", _i32)]


class PatchMap(C.Structure):
    _fields_ = [("patch_block", _ptr), ("block_patch", _ptr)]


class TagParams(C.Structure):
    _fields_ = [("dx", _dbl), ("gradient_threshold", _dbl), ("radial_gradient_threshold", _dbl),
                ("n_error_buf", _i32), ("block", _i32)]


class EnsembleC(C.Structure):
    _fields_ = [("dtype", _i32), ("nboxes", _i32), ("dims", C.POINTER(_i32)), ("dx", _dbl), ("state", _ptr),
                ("work", _ptr), ("table", _ptr), ("state_bytes", _i64), ("work_bytes", _i64),
                ("table_bytes", _i64)]


class EnsembleBox(C.Structure):
    _fields_ = [("base", _i64), ("jstride", _i64), ("kstride", _i64), ("x_offset", _i32), ("y_offset", _i32)]


class EnsemblePlan(C.Structure):
    _fields_ = [("tile_config", _i32), ("z_chunk", _i32), ("n_items", _i64), ("grid_a", _i32), ("grid_b", _i32),
                ("plane_elems", _i64), ("key", _u64)]


# name -> (restype, argtypes); every symbol here is declared in include/axs.h
SIGNATURES = {
    "axs_background_eval": (_i32, [C.POINTER(BackgroundC), _dbl, C.POINTER(BackgroundValues)]),
    "axs_background_rhs_coeffs": (_i32, [C.POINTER(BackgroundC), _dbl, C.POINTER(RhsCoeffs)]),
    "axs_background_tau_from_log_mr_over_h": (_i32, [C.POINTER(BackgroundC), _dbl, C.POINTER(_dbl)]),
    "axs_xi_from_comoving_length": (_dbl, [_dbl, _dbl, _dbl, _dbl]),
    "axs_xi_from_plaquette_count": (_dbl, [_dbl, _dbl, _dbl, _dbl, _dbl]),
    "axs_plaquette_count_for_target_xi": (_dbl, [_dbl, C.c_int, _dbl, _dbl, _dbl]),
    "axs_status_string": (C.c_char_p, [C.c_int]),
    "axs_last_error": (C.c_char_p, []),
    "axs_abi_version": (C.c_int, []),
    "axs_set_device_wait_polls": (_i32, [C.c_uint32, C.POINTER(C.c_uint32)]),
    "axs_count_nonfinite": (_i32, [C.POINTER(Fab), _ptr, _ptr]),
    "axs_level_count_nonfinite": (_i32, [C.POINTER(LevelC), _ptr, _ptr]),
    "axs_eval_rhs": (_i32, [C.POINTER(Fab), C.POINTER(Fab), _dbl, C.POINTER(RhsCoeffs), _ptr]),
    "axs_fill_periodic_ghosts": (_i32, [C.POINTER(Fab), _ptr]),
    "axs_fill_periodic_ghosts_xy": (_i32, [C.POINTER(Fab), _ptr]),
    "axs_fab_pack_z_planes": (_i32, [C.POINTER(Fab), _i32, _i32, _ptr, _ptr]),
    "axs_fab_unpack_z_planes": (_i32, [C.POINTER(Fab), _i32, _i32, _ptr, _ptr]),
    "axs_lincomb": (_i32, [C.POINTER(Fab), C.POINTER(Fab), _dbl, C.POINTER(Fab), _ptr]),
    "axs_rk4_combine": (_i32, [C.POINTER(Fab)] * 6 + [_dbl, _ptr]),
    "axs_level_layout_for": (_i32, [_i32, _i32, _i32, _i32, C.POINTER(LevelLayout)]),
    "axs_level_tile_config_count": (C.c_int, [_i32]),
    "axs_level_tile_config_name": (C.c_char_p, [_i32, _i32]),
    "axs_level_fill_ghosts": (_i32, [C.POINTER(LevelC), _ptr]),
    "axs_level_import_fab": (_i32, [C.POINTER(LevelC), C.POINTER(Fab), _ptr]),
    "axs_level_export_fab": (_i32, [C.POINTER(LevelC), C.POINTER(Fab), _ptr]),
    "axs_level_upload": (_i32, [C.POINTER(LevelC), _ptr, _ptr]),
    "axs_level_download": (_i32, [C.POINTER(LevelC), _ptr, _ptr]),
    "axs_level_rk4_advance": (_i32, [C.POINTER(LevelC), C.POINTER(BackgroundC), _dbl, _dbl, _dbl, _i32, _ptr]),
    "axs_level_rk4_sweep": (_i32, [C.POINTER(LevelC), C.POINTER(BackgroundC), _dbl, _dbl, _dbl, _i32, _ptr]),
    "axs_level_rk4_step_to": (_i32, [C.POINTER(LevelC), _ptr, C.POINTER(BackgroundC), _dbl, _dbl, _dbl, _ptr]),
    "axs_level_device_status": (_i32, [C.POINTER(LevelC), _ptr]),
    "axs_level_handoff_rescale": (_i32, [C.POINTER(LevelC), _dbl, _dbl, _dbl, _dbl, _ptr]),
    "axs_level_adjoint_work_bytes": (_i32, [_i32, _i32, _i32, _i32, C.POINTER(_i64)]),
    "axs_level_rk4_adjoint_step": (_i32, [C.POINTER(LevelC), _ptr, _ptr, _i64, C.POINTER(BackgroundC), _dbl, _dbl,
                                          _dbl, _ptr, _ptr]),
    "axs_level_string_core_loss": (_i32, [C.POINTER(LevelC), _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr]),
    "axs_diagnostics_scratch_bytes": (_i32, [_i32, _i32, _i32, C.POINTER(_i64)]),
    "axs_diagnostics": (_i32, [C.POINTER(Fab), C.POINTER(DiagParams), _ptr, _ptr, _ptr, _i64, _ptr, _i64, _ptr]),
    "axs_level_diagnostics": (_i32, [C.POINTER(LevelC), C.POINTER(DiagParams), _ptr, _ptr, _ptr, _i64, _ptr, _i64,
                                     _ptr]),
    "axs_diagnostics_static_scratch": (_i32, [C.POINTER(Fab), C.POINTER(DiagParams), _ptr, _ptr, _ptr, _i64, _ptr]),
    "axs_patches_layout": (_i32, [_i32, _i32, _i32, C.POINTER(PatchLayout)]),
    "axs_patches_init": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchPlan), _ptr]),
    "axs_patches_fill": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchMap), C.POINTER(LevelC), C.POINTER(LevelC), _dbl,
                                _dbl, _i32, _ptr]),
    "axs_patches_fill_list": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchMap), C.POINTER(LevelC), C.POINTER(LevelC),
                                     _dbl, _dbl, _i32, _ptr, _i32, _ptr]),
    "axs_patches_copy_boxes": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchesC), _ptr, _ptr]),
    "axs_patches_rk4_step": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchPlan), C.POINTER(BackgroundC), _dbl, _dbl,
                                    _dbl, _ptr]),
    "axs_patches_average_down": (_i32, [C.POINTER(PatchesC), C.POINTER(PatchMap), C.POINTER(LevelC), _ptr]),
    "axs_patches_device_status": (_i32, [C.POINTER(PatchesC), _ptr]),
    "axs_patches_diagnostics_scratch_bytes": (_i32, [_i32, _i32, C.POINTER(_i64)]),
    "axs_patches_diagnostics": (_i32, [C.POINTER(PatchesC), C.POINTER(DiagParams), _ptr, _ptr, _i64, _ptr, _i64,
                                       _ptr]),
    "axs_level_masked_a_dot": (_i32, [C.POINTER(LevelC), _i32, _dbl, _dbl, _ptr, _ptr, _ptr, _i64, _ptr]),
    "axs_spectrum_scratch_bytes": (_i32, [_i32, _i32, _i32, C.POINTER(_i64)]),
    "axs_spectrum_bin": (_i32, [_ptr, _i32, _i32, _i32, _i32, _ptr, _ptr, _ptr, _ptr, _i64, _ptr]),
    "axs_tag_scratch_bytes": (_i32, [_i32, _i32, _i32, C.POINTER(_i64)]),
    "axs_level_tag_cells": (_i32, [C.POINTER(LevelC), C.POINTER(TagParams), _ptr, _ptr, _ptr, _ptr, _i64, _ptr]),
    "axs_ensemble_sizes": (_i32, [_i32, _i32, C.POINTER(_i32), C.POINTER(_i64), C.POINTER(_i64), C.POINTER(_i64)]),
    "axs_ensemble_box_layout": (_i32, [_i32, _i32, C.POINTER(_i32), _i32, C.POINTER(EnsembleBox)]),
    "axs_ensemble_tile_config_count": (_i32, [_i32]),
    "axs_ensemble_tile_config_name": (C.c_char_p, [_i32, _i32]),
    "axs_ensemble_init": (_i32, [C.POINTER(EnsembleC), C.POINTER(EnsemblePlan), _ptr]),
    "axs_ensemble_fill_ghosts": (_i32, [C.POINTER(EnsembleC), _ptr]),
    "axs_ensemble_rk4_advance": (_i32, [C.POINTER(EnsembleC), C.POINTER(EnsemblePlan), C.POINTER(BackgroundC), _dbl,
                                        _dbl, _dbl, _i32, _ptr]),
    "axs_ensemble_diagnostics_scratch_bytes": (_i32, [_i32, C.POINTER(_i32), C.POINTER(_i64)]),
    "axs_ensemble_diagnostics": (_i32, [C.POINTER(EnsembleC), C.POINTER(DiagParams), _ptr, _ptr, _i64, _ptr]),
    "axs_ensemble_device_status": (_i32, [C.POINTER(EnsembleC), _ptr]),
    "axs_plaquette_winding_batch": (_i32, [_ptr, _i64, _ptr, _ptr]),
    "axs_fourier_spectrum": (_i32, [_ptr, _i32, _i32, _i32, _dbl, _u64, _i32, _ptr]),
}


class AxsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[axs status {status}] {message}")
        self.status = status


_lib = None


def lib():
    """Load libaxs_gb300.so (building it first if the sources are newer)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from ._build import build
            build()
        try:
            L = C.CDLL(LIB_PATH)
        except OSError as e:  # pragma: no cover - loud failure by design
            raise RuntimeError(f"cannot load the axion-string CUDA library {LIB_PATH}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.axs_abi_version() != 2:
            raise RuntimeError("libaxs_gb300.so ABI version mismatch")
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != AXS_OK:
        msg = lib().axs_last_error().decode(errors="replace")
        raise AxsError(status, msg or lib().axs_status_string(status).decode())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def set_device_wait_polls(polls: int) -> int:
    """Polls a bounded device-side wait makes before it gives up (0: at once,
    for testing the timeout path); returns the previous value."""
    prev = C.c_uint32()
    call("axs_set_device_wait_polls", int(polls), C.byref(prev))
    return prev.value
