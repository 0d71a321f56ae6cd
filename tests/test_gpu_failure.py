"""Failure detection without a GPU fault.

Bounded device waits: with the library's wait limit set to 0 polls every
bounded wait of the stencil kernels gives up at once. The kernel then records
the timeout in the level's status word, waits (with its own fixed bound) for
the copies it has in flight and ends, so the context stays usable: the status
call reports AXS_ERR_DEVICE_TIMEOUT, and with the limit restored the next
steps are bit for bit those of a level that never timed out.

Non-finite cells: NaN and infinite values planted from the host are counted
per cell, on a level and on a FAB."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _state(n, seed, dtype):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((4, n, n, n))
    v[:2] += 2.0
    return torch.from_numpy(v).to(dtype)


@pytest.mark.parametrize("dtype,tiling", [(torch.float32, "f32 v2 64x8 ring8"),
                                          (torch.float32, "f32 fused 32x16 ring6 t640"),
                                          (torch.float32, "f32 fused 32x16 ring7 t640"),
                                          (torch.float64, None)])
def test_expired_waits_are_reported_and_the_level_recovers(axs, dtype, tiling):
    L = axs._lib
    n, bg = 64, axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    v = _state(n, 3, dtype).cuda()
    lv = axs.PeriodicLevel(n, 0.5, dtype=dtype)
    if tiling:
        lv.tile_config = [cid for cid, name in lv.tile_configs() if name == tiling][0]
    lv.set_state(v)
    prev = L.set_device_wait_polls(0)
    try:
        lv.advance(bg, 1.0, 0.0, 0.1, 2)
        torch.cuda.synchronize()
    finally:
        L.set_device_wait_polls(prev)
    with pytest.raises(L.AxsError) as err:
        lv.device_status()
    assert err.value.status == L.AXS_ERR_DEVICE_TIMEOUT
    lv.device_status()  # the status word was cleared by the report
    # the context is usable and the next run is exact
    lv.set_state(v)
    lv.advance(bg, 1.0, 0.0, 0.1, 3)
    lv.device_status()
    ref = axs.PeriodicLevel(n, 0.5, dtype=dtype)
    ref.tile_config = lv.tile_config
    ref.set_state(v)
    ref.advance(bg, 1.0, 0.0, 0.1, 3)
    ref.device_status()
    assert torch.equal(lv.state, ref.state)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_nonfinite_cells_are_counted(axs, dtype):
    n = 24
    v = _state(n, 5, dtype)
    clean = v.clone()
    bad = [((0, 1, 2, 3), np.nan), ((2, 5, 5, 5), np.inf), ((3, 5, 5, 5), np.nan),  # one cell, two components
           ((1, 23, 0, 17), -np.inf), ((2, 7, 23, 0), np.nan)]
    for idx, val in bad:
        v[idx] = val
    lv = axs.PeriodicLevel(n, 0.5, dtype=dtype)
    lv.set_state(clean.cuda())
    assert lv.count_nonfinite() == 0
    lv.set_state(v.cuda())
    assert lv.count_nonfinite() == 4
    lvl = axs.AxionStringsLevel(n, 0.5, axs.Background.expanding(2.0, 1.0, lambda0=2.0), dtype=dtype)
    lvl.level.set_state(v.cuda())
    with pytest.raises(FloatingPointError):
        lvl.check_finite()
    # the FAB entry point on the same cells (ghosts hold finite garbage that must not count)
    t = axs.new_fab((n, n, n), 2, dtype=dtype)
    t.fill_(1e300 if dtype == torch.float64 else 1e30)
    axs.valid(t, 2).copy_(v.cuda())
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    import ctypes as C
    axs._lib.call("axs_count_nonfinite", C.byref(axs.fab(t, 2)), cnt.data_ptr(), None)
    assert int(cnt.item()) == 4
