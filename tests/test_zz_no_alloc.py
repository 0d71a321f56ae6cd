"""The allocation-free diagnostics entry point, for host codes that cannot give
this library device memory (e.g. an application whose arena owns the GPU).

axs_diagnostics_static_scratch must return what axs_diagnostics returns with
caller-provided scratch, call after call. Consecutive calls switch between the
pass's modes (the fused pass, the string finder alone, the split FP32
per-cell pass), whose kernels fill different fields of the per-block records
in the shared static array, so a record left over from the previous call in
another mode would show. A 128^3 box uses the largest grid the pass launches
(8 blocks per SM). Kept in its own file, collected last, and independent of
the other tests' state.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# (want_energy, want_plaquettes, want_velocity, per_cell_fp32)
MODES = {"fused": (1, 1, 1, 0), "strings": (0, 1, 0, 0), "fp32cell": (1, 1, 1, 1)}


def _read(L, res):
    return L.DiagResult.from_buffer_copy(res.cpu().numpy().tobytes())


def _box(A, n, dtype, seed):
    rng = np.random.default_rng(seed)
    st = rng.standard_normal((4, n[2], n[1], n[0])) * np.array([1.0, 1.0, 0.3, 0.3])[:, None, None, None]
    t = A.new_fab(n, 2, dtype=dtype)
    A.valid(t, 2).copy_(torch.from_numpy(st).to(dtype).cuda())
    A.fill_periodic_ghosts(t, 2)
    return t


def _compare(A, n, dtype, calls):
    """calls: [(mode, seed), ...] run back to back through both entry points."""
    L = A._lib
    lib = L.lib()
    stream = torch.cuda.current_stream().cuda_stream
    ncell = n[0] * n[1] * n[2]
    ref_res = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device="cuda")
    ref_list = torch.full((3 * ncell,), -1, dtype=torch.int64, device="cuda")
    scratch = torch.zeros(A.level.scratch_bytes(*n), dtype=torch.uint8, device="cuda")
    res = torch.zeros_like(ref_res)
    lst = torch.full_like(ref_list, -1)
    for mode, seed in calls:
        params = L.DiagParams(0.5, 1.1, 1.3, 0.4, 1.14, L.MASK_A, 0.8, L.BOUNDARY_GHOSTS, *MODES[mode])
        t = _box(A, n, dtype, seed)
        f = A.fab(t, 2)
        assert lib.axs_diagnostics(C.byref(f), C.byref(params), None, ref_res.data_ptr(), ref_list.data_ptr(),
                                   ref_list.numel(), scratch.data_ptr(), scratch.numel(), stream) == L.AXS_OK
        assert lib.axs_diagnostics_static_scratch(C.byref(f), C.byref(params), None, res.data_ptr(),
                                                  lst.data_ptr(), lst.numel(), stream) == L.AXS_OK, \
            lib.axs_last_error()
        torch.cuda.synchronize()
        a, b = _read(L, ref_res), _read(L, res)
        assert b.status == L.AXS_OK and a.status == L.AXS_OK
        assert (b.n_p_plain, b.n_p_weighted, b.vel_count, b.n_listed) == \
            (a.n_p_plain, a.n_p_weighted, a.vel_count, a.n_listed), mode
        assert a.n_p_plain > 0, "the box should hold pierced plaquettes"
        np.testing.assert_allclose(list(b.energy_sums), list(a.energy_sums), rtol=1e-12, atol=0)
        assert b.vel_sum == pytest.approx(a.vel_sum, rel=1e-12)
        np.testing.assert_array_equal(np.sort(lst[: b.n_listed].cpu().numpy()),
                                      np.sort(ref_list[: a.n_listed].cpu().numpy()))


def _lib_or_skip():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import axion_strings_adaptive_gb300 as A
    A.build()
    return A


@pytest.mark.parametrize("dtype,calls", [
    (torch.float64, [("fused", 7), ("fused", 8)]),
    (torch.float64, [("fused", 9), ("strings", 10)]),
    (torch.float64, [("strings", 11), ("fused", 12)]),
    (torch.float32, [("fused", 7), ("fused", 8)]),
    (torch.float32, [("strings", 13), ("fp32cell", 14)]),
    (torch.float32, [("fp32cell", 15), ("fused", 16)]),
])
def test_static_scratch_matches_caller_scratch(dtype, calls):
    _compare(_lib_or_skip(), (24, 20, 18), dtype, calls)


@pytest.mark.parametrize("dtype,calls", [
    (torch.float32, [("fp32cell", 21), ("fused", 22)]),
    (torch.float64, [("fused", 23), ("strings", 24)]),
])
def test_static_scratch_full_grid(dtype, calls):
    _compare(_lib_or_skip(), (128, 128, 128), dtype, calls)
