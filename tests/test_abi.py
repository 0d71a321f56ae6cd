"""C-ABI checks that need no GPU: the library loads, exports exactly the entry
points include/axs.h declares, and its host-side scalar models (background
coefficients, xi) reproduce the reference-generated golden vectors. Argument
validation happens before any CUDA call, so bad descriptors are rejected here
too."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "axs.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(axs_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def L():
    from axion_strings_adaptive_gb300 import _build, _lib
    _build.build()
    return _lib


def test_every_declared_symbol_is_exported(L):
    lib = L.lib()
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), f"{n} declared in axs.h but not exported"
    # and the Python binding covers every declaration
    assert set(names) == set(L.SIGNATURES), set(names) ^ set(L.SIGNATURES)


def test_abi_version_and_status_strings(L):
    lib = L.lib()
    assert lib.axs_abi_version() == 2
    for s in range(8):
        assert lib.axs_status_string(s)


def test_background_matches_reference(L, golden):
    from axion_strings_adaptive_gb300 import Background
    g = golden("kats.npz")
    for cfg, rows in zip(g["bg_cfg"], g["bg_out"]):
        bg = Background.expanding(cfg[0], cfg[1], c1=cfg[2], tau_switch=cfg[3], has_switch=bool(cfg[4]))
        for tau, row in zip(g["bg_tau"], rows):
            v = bg.values(tau)
            np.testing.assert_allclose([v.R, v.R_prime, v.kappa, v.lambda_, v.H], row[:5], rtol=2e-15)
            assert v.H / v.m_r == pytest.approx(row[5], rel=1e-14)
    for (a_inv, c0, l), tau in zip(g["bg_log_in"], g["bg_log_tau"]):
        assert Background.expanding(a_inv, c0).tau_from_log_mr_over_h(l) == pytest.approx(tau, rel=1e-15)
    for a, m in enumerate((1.0, 2.3, 0.7)):
        v = Background.flat(m).values(1.0)
        np.testing.assert_array_equal([v.R, v.R_prime, v.kappa, v.lambda_], g["flat_out"][a, 0])
    for a, gp in enumerate((0.5, 1.0, 3.0)):
        for b, t in enumerate((-2.0, -0.3, 0.0, 0.7, 4.0)):
            v = Background.pre_evolution(gp).values(t)
            np.testing.assert_allclose([v.R, v.R_prime, v.kappa, v.lambda_], g["pre_out"][a, b, :4], rtol=1e-15)


def test_lambda_scale_and_handoff_blend(L):
    from axion_strings_adaptive_gb300 import Background
    b1 = Background.expanding(2.0, 1.0)
    b2 = Background.expanding(2.0, 1.0, lambda0=2.0)
    for tau in (1.0, 2.5, 7.0):
        assert b2.lambda_(tau) == pytest.approx(2.0 * b1.lambda_(tau), rel=1e-15)
    # smoothstep blend away from frozen pre-evolution values (AxionStringsLevel.cpp:893-906)
    import dataclasses
    bb = dataclasses.replace(b1, blend_dtau=2.0, blend_tau_start=1.0, blend_lambda_start=5.0, blend_curv_start=0.3)
    c0 = bb.rhs_coeffs(1.0)
    assert c0.lambda_ == pytest.approx(5.0) and c0.kappa == pytest.approx(0.3)
    cm = bb.rhs_coeffs(2.0)  # t = 0.5 -> s = 0.5
    assert cm.lambda_ == pytest.approx(0.5 * 5.0 + 0.5 * b1.lambda_(2.0))
    c1 = bb.rhs_coeffs(3.5)
    assert c1.lambda_ == pytest.approx(b1.lambda_(3.5), rel=1e-15)


def test_xi_matches_reference(L, golden):
    from axion_strings_adaptive_gb300 import (plaquette_count_for_target_xi, xi_from_comoving_length,
                                              xi_from_plaquette_count)
    g = golden("kats.npz")
    for x, xi, xil, inv in zip(g["xi_in"], g["xi_out"], g["xi_len_out"], g["xi_inv_out"]):
        assert xi_from_plaquette_count(*x) == xi
        assert xi_from_comoving_length((2 / 3) * x[0] * x[1], *x[2:]) == xil
        assert plaquette_count_for_target_xi(0.7, 64, x[2], x[3], x[4]) == inv


def test_validation_rejects_bad_input_without_gpu(L):
    lib = L.lib()
    c = L.RhsCoeffs(0.0, 1.0, 1.0)
    f = L.Fab(None, L.AXS_F64, 8, 8, 8, 2, 4, 12, 144, 1728)
    assert lib.axs_eval_rhs(C.byref(f), C.byref(f), 0.5, C.byref(c), None) == L.AXS_ERR_INVALID_ARGUMENT
    assert b"null data" in lib.axs_last_error()
    f2 = L.Fab(C.c_void_p(256), L.AXS_F64, 8, 8, 8, 2, 4, 11, 144, 1728)  # jstride too small
    assert lib.axs_eval_rhs(C.byref(f2), C.byref(f2), 0.5, C.byref(c), None) == L.AXS_ERR_INVALID_ARGUMENT
    assert b"strides" in lib.axs_last_error()
    f3 = L.Fab(C.c_void_p(256), 7, 8, 8, 8, 2, 4, 12, 144, 1728)
    assert lib.axs_eval_rhs(C.byref(f3), C.byref(f3), 0.5, C.byref(c), None) == L.AXS_ERR_INVALID_ARGUMENT
    lay = L.LevelLayout()
    assert lib.axs_level_layout_for(L.AXS_F32, 6, 8, 8, C.byref(lay)) == L.AXS_ERR_UNSUPPORTED  # nx % 4
    assert lib.axs_level_layout_for(L.AXS_F32, 8, 1, 8, C.byref(lay)) == L.AXS_ERR_UNSUPPORTED  # ny >= 2
    assert lib.axs_level_layout_for(L.AXS_F64, 6, 8, 8, C.byref(lay)) == L.AXS_OK
    # x = 0 on a 128-byte line (16 doubles), rows a whole number of lines
    assert lay.x_offset == 16 and lay.y_offset == 2 and lay.jstride == 32
    assert lay.kstride == 32 * 12 and lay.cstride == 32 * 12 * 8
    assert lay.state_bytes == 4 * lay.cstride * 8 and lay.work_bytes == 8 * lay.cstride * 8 + 256
    assert lib.axs_level_layout_for(L.AXS_F32, 512, 512, 512, C.byref(lay)) == L.AXS_OK
    assert lay.x_offset == 32 and lay.jstride == 576 and (lay.jstride * 4) % 128 == 0
    assert lib.axs_level_tile_config_count(L.AXS_F32) >= 1 and lib.axs_level_tile_config_count(L.AXS_F64) >= 1
    assert lib.axs_level_tile_config_name(L.AXS_F32, 0) == lib.axs_level_tile_config_name(L.AXS_F32, 1)
    assert lib.axs_level_tile_config_name(L.AXS_F32, 99) is None
    lv = L.LevelC(None, None, L.AXS_F32, 8, 8, 8, 0.5, 0)
    bg = L.BackgroundC(0, 0, 2.0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0)
    assert lib.axs_level_rk4_advance(C.byref(lv), C.byref(bg), 1.0, 0.0, 0.1, 1, None) == L.AXS_ERR_INVALID_ARGUMENT
    lv2 = L.LevelC(C.c_void_p(4096), C.c_void_p(8192), L.AXS_F32, 8, 8, 8, 0.5, 0)
    assert lib.axs_level_rk4_advance(C.byref(lv2), C.byref(bg), 1.0, 0.0, -0.1, 1, None) == L.AXS_ERR_INVALID_ARGUMENT
    bad_bg = L.BackgroundC(0, 0, 0.5, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0)  # a_inv <= 1
    assert lib.axs_level_rk4_advance(C.byref(lv2), C.byref(bad_bg), 1.0, 0.0, 0.1, 1, None) == \
        L.AXS_ERR_INVALID_ARGUMENT
    assert lib.axs_level_rk4_advance(C.byref(lv2), C.byref(bg), 1.0, 0.0, 0.1, 0, None) == L.AXS_OK  # no-op
    lv3 = L.LevelC(C.c_void_p(4096 + 16), C.c_void_p(8192), L.AXS_F32, 8, 8, 8, 0.5, 0)
    assert lib.axs_level_rk4_advance(C.byref(lv3), C.byref(bg), 1.0, 0.0, 0.1, 1, None) == L.AXS_ERR_ALIGNMENT
    b = C.c_int64()
    assert lib.axs_diagnostics_scratch_bytes(0, 8, 8, C.byref(b)) == L.AXS_ERR_INVALID_ARGUMENT
    assert lib.axs_plaquette_winding_batch(None, -1, None, None) == L.AXS_ERR_INVALID_ARGUMENT
    assert lib.axs_plaquette_winding_batch(None, 0, None, None) == L.AXS_OK


def test_package_refuses_cpu_tensors():
    import torch

    import axion_strings_adaptive_gb300 as A
    with pytest.raises(ValueError, match="CUDA"):
        A.fab(torch.zeros((4, 8, 8, 8)), 2)


def test_ensemble_layout_and_validation(L):
    lib = L.lib()
    dims = [32, 32, 32, 48, 40, 24, 16, 16, 8]
    arr = (C.c_int32 * len(dims))(*dims)
    sb, wb, tb = C.c_int64(), C.c_int64(), C.c_int64()
    L.call("axs_ensemble_sizes", L.AXS_F32, 3, arr, C.byref(sb), C.byref(wb), C.byref(tb))
    plane = sb.value // 16
    assert wb.value == 2 * sb.value and tb.value > 128
    end = 0
    for b in range(3):
        lay = L.EnsembleBox()
        L.call("axs_ensemble_box_layout", L.AXS_F32, 3, arr, b, C.byref(lay))
        nx, ny, nz = dims[3 * b:3 * b + 3]
        ref = L.LevelLayout()
        L.call("axs_level_layout_for", L.AXS_F32, nx, ny, nz, C.byref(ref))
        assert (lay.jstride, lay.kstride, lay.x_offset, lay.y_offset) == \
               (ref.jstride, ref.kstride, ref.x_offset, ref.y_offset)
        assert lay.base % 32 == 0 and lay.base >= end  # 128-byte aligned, no overlap
        end = lay.base + nz * lay.kstride
    assert end <= plane
    assert lib.axs_ensemble_tile_config_count(L.AXS_F32) >= 3
    assert lib.axs_ensemble_tile_config_name(L.AXS_F32, 0)
    assert lib.axs_ensemble_tile_config_name(L.AXS_F32, 99) is None
    # rejected before any CUDA call
    bad = (C.c_int32 * 3)(30, 32, 32)  # nx not a multiple of 4 (FP32 rows)
    assert lib.axs_ensemble_sizes(L.AXS_F32, 1, bad, C.byref(sb), C.byref(wb), C.byref(tb)) == L.AXS_ERR_UNSUPPORTED
    assert lib.axs_ensemble_sizes(L.AXS_F32, 0, arr, C.byref(sb), C.byref(wb), C.byref(tb)) == \
        L.AXS_ERR_INVALID_ARGUMENT
    e = L.EnsembleC(L.AXS_F32, 3, arr, 0.5, None, None, None, 0, 0, 0)
    plan = L.EnsemblePlan()
    assert lib.axs_ensemble_init(C.byref(e), C.byref(plan), None) == L.AXS_ERR_INVALID_ARGUMENT
    e2 = L.EnsembleC(L.AXS_F32, 3, arr, 0.5, 128, 128, 128, 16, 16, 16)  # buffers too small
    assert lib.axs_ensemble_init(C.byref(e2), C.byref(plan), None) == L.AXS_ERR_WORKSPACE


def test_cpp_host_demo_is_built(L):
    import subprocess
    from axion_strings_adaptive_gb300 import _build
    r = subprocess.run([_build.DEMO_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr


def test_patch_layout_rows_arenas_and_counts(L):
    """Patch rows are whole 32-byte sectors (n + 16 columns), boxes start on
    128-byte lines, patch sizes the fused step takes need no work arena (and
    their count is not tied to a grid dimension); the two-sweep sizes keep
    their work arena."""
    lib = L.lib()
    lay = L.PatchLayout()
    assert lib.axs_patches_layout(L.AXS_F32, 32, 60000, C.byref(lay)) == L.AXS_OK
    assert lay.jstride == 48 and lay.kstride == 48 * 40 and lay.patch_elems == 48 * 40 * 40
    assert (lay.patch_elems * 4) % 128 == 0 and lay.plane_elems == 60000 * lay.patch_elems
    assert lay.work_bytes == 0 and lay.state_bytes == 4 * lay.plane_elems * 4
    assert lib.axs_patches_layout(L.AXS_F64, 32, 1000, C.byref(lay)) == L.AXS_OK
    assert lay.jstride == 48 and lay.work_bytes == 0
    assert lib.axs_patches_layout(L.AXS_F32, 16, 1000, C.byref(lay)) == L.AXS_OK  # two-sweep size
    assert lay.jstride == 32 and lay.work_bytes == 8 * lay.plane_elems * 4
    assert lib.axs_patches_layout(L.AXS_F32, 32, 70000, C.byref(lay)) == L.AXS_OK  # fused: launched in chunks
    assert lib.axs_patches_layout(L.AXS_F32, 32, (1 << 22) + 1, C.byref(lay)) == L.AXS_ERR_INVALID_ARGUMENT
    # a two-sweep patch set needs its work arena
    p = L.PatchesC(L.AXS_F32, 16, 10, 0.25, C.c_void_p(1 << 20), None, C.c_void_p(1 << 21), 1 << 30, 0, 1 << 30)
    plan = L.PatchPlan()
    assert lib.axs_patches_init(C.byref(p), C.byref(plan), None) == L.AXS_ERR_INVALID_ARGUMENT


def test_device_wait_polls_setting_round_trips(L):
    lib = L.lib()
    prev = C.c_uint32()
    assert lib.axs_set_device_wait_polls(123, C.byref(prev)) == L.AXS_OK
    assert prev.value == L.AXS_DEFAULT_WAIT_POLLS
    assert L.set_device_wait_polls(L.AXS_DEFAULT_WAIT_POLLS) == 123
    assert lib.axs_set_device_wait_polls(L.AXS_DEFAULT_WAIT_POLLS, None) == L.AXS_OK


def test_nonfinite_count_validates_arguments(L):
    lib = L.lib()
    assert lib.axs_count_nonfinite(None, None, None) == L.AXS_ERR_INVALID_ARGUMENT
    assert lib.axs_level_count_nonfinite(None, None, None) == L.AXS_ERR_INVALID_ARGUMENT


def test_diagnostics_rejects_small_scratch_without_gpu(L):
    """The scratch check runs before any launch: AXS_ERR_WORKSPACE, nothing
    dereferenced (the data pointer is never touched)."""
    lib = L.lib()
    f = L.Fab(C.c_void_p(4096), L.AXS_F32, 8, 8, 8, 2, 4, 12, 144, 1728)
    p = L.DiagParams(0.5, 1.0, 2.0, 0.1, 1.0, L.MASK_NONE, 0.8, L.BOUNDARY_GHOSTS, 1, 1, 1, 0)
    need = C.c_int64()
    assert lib.axs_diagnostics_scratch_bytes(8, 8, 8, C.byref(need)) == L.AXS_OK and need.value > 16
    rc = lib.axs_diagnostics(C.byref(f), C.byref(p), None, C.c_void_p(8192), None, 0, C.c_void_p(16384), 16, None)
    assert rc == L.AXS_ERR_WORKSPACE
    assert b"scratch too small" in lib.axs_last_error()


def test_step_to_validates_its_destination_without_gpu(L):
    lib = L.lib()
    lv = L.LevelC(C.c_void_p(4096), C.c_void_p(1 << 20), L.AXS_F32, 8, 8, 8, 0.5, 0)
    bg = L.BackgroundC(0, 0, 2.0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0)
    assert lib.axs_level_rk4_step_to(C.byref(lv), None, C.byref(bg), 1.0, 0.0, 0.1, None) == \
        L.AXS_ERR_INVALID_ARGUMENT
    assert lib.axs_level_rk4_step_to(C.byref(lv), C.c_void_p(4096), C.byref(bg), 1.0, 0.0, 0.1, None) == \
        L.AXS_ERR_INVALID_ARGUMENT
    assert b"overlaps the state" in lib.axs_last_error()
    assert lib.axs_level_rk4_step_to(C.byref(lv), C.c_void_p((1 << 20) + 128), C.byref(bg), 1.0, 0.0, 0.1, None) == \
        L.AXS_ERR_INVALID_ARGUMENT
    assert b"overlaps the work" in lib.axs_last_error()
    assert lib.axs_level_rk4_step_to(C.byref(lv), C.c_void_p((1 << 24) + 16), C.byref(bg), 1.0, 0.0, 0.1, None) == \
        L.AXS_ERR_ALIGNMENT


def test_level_flags_are_checked_without_gpu(L):
    lib = L.lib()
    bg = L.BackgroundC(0, 0, 2.0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0)
    lv = L.LevelC(C.c_void_p(4096), C.c_void_p(8192), L.AXS_F32, 8, 8, 8, 0.5, 0, 4)
    assert lib.axs_level_rk4_advance(C.byref(lv), C.byref(bg), 1.0, 0.0, 0.1, 1, None) == L.AXS_ERR_INVALID_ARGUMENT
    assert b"unknown level flags" in lib.axs_last_error()
    lv.flags = L.LEVEL_COMPENSATED_FP32
    assert lib.axs_level_rk4_advance(C.byref(lv), C.byref(bg), 1.0, 0.0, 0.1, 0, None) == L.AXS_OK  # no-op
