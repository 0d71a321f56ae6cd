"""Ensemble (batching) path through the C ABI: boxes of uneven sizes packed in
one arena and advanced by one persistent launch per sweep evolve bit for bit
as the same boxes advanced one level at a time, for every compiled tiling and
z-chunk target; per-box diagnostics equal the level diagnostics; a captured
CUDA graph replays the eager run exactly."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu

DIMS = [(32, 32, 32), (48, 40, 24), (64, 16, 36), (24, 28, 12), (16, 16, 8)]


def _box_ic(dims, seed, dtype):
    from axion_strings_adaptive_gb300 import ic
    nx, ny, nz = dims
    s = torch.zeros((4, nz, ny, nx), dtype=torch.float64, device="cuda")
    for c in (0, 1):
        s[c] = ic.fourier_component(dims, max(2.0, min(dims) / 4), seed, c).cuda()
    g = torch.Generator(device="cuda").manual_seed(seed)
    s[2:] = 0.1 * torch.randn((2, nz, ny, nx), generator=g, device="cuda", dtype=torch.float64)
    return s.to(dtype)


def _levels(axs, dims, dtype, bg, steps):
    out = []
    for b, d in enumerate(dims):
        lv = axs.PeriodicLevel(d, 0.5, dtype=dtype)
        lv.set_state(_box_ic(d, 100 + b, dtype))
        lv.advance(bg, 1.0, 0.0, 0.1, steps)
        lv.device_status()
        out.append(lv)
    return out


def _ensemble(axs, dims, dtype):
    e = axs.Ensemble(dims, 0.5, dtype=dtype)
    for b, d in enumerate(dims):
        e.set_box(b, _box_ic(d, 100 + b, dtype))
    e.fill_ghosts()
    return e


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_ensemble_matches_levels_bitwise_every_tiling(axs, dtype):
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    steps = 4
    ref = [lv.get_state() for lv in _levels(axs, DIMS, dtype, bg, steps)]
    e = _ensemble(axs, DIMS, dtype)
    init = e.state.clone()
    for cid, name in e.tile_configs():
        for zc in (0, 3, 7):
            e.state.copy_(init)
            e.init(cid, zc)
            e.advance(bg, 1.0, 0.0, 0.1, steps)
            e.device_status()
            for b in range(len(DIMS)):
                assert torch.equal(e.get_box(b), ref[b]), (name, zc, b)


def test_ensemble_diagnostics_match_levels(axs):
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    levels = _levels(axs, DIMS, torch.float32, bg, 6)
    e = _ensemble(axs, DIMS, torch.float32)
    e.advance(bg, 1.0, 0.0, 0.1, 6)
    got = e.diagnostics(bg, 1.6)
    for b, lv in enumerate(levels):
        ref = lv.diagnostics(bg, 1.6, want_list=False)
        assert (got[b].n_p_plain, got[b].n_p_weighted, got[b].vel_count) == \
               (ref.n_p_plain, ref.n_p_weighted, ref.vel_count)
        assert got[b].energy == ref.energy
        assert got[b].mean_gamma_sq_v_sq == ref.mean_gamma_sq_v_sq


def test_graph_replay_equals_eager(axs):
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    e = _ensemble(axs, DIMS, torch.float32)
    init = e.state.clone()
    e.advance(bg, 1.0, 0.0, 0.1, 8)
    eager = e.diagnostics(bg, 1.8)
    eager_state = e.state.clone()
    e.state.copy_(init)
    g = e.capture(bg, 1.0, 0.0, 0.1, 8)
    assert torch.equal(e.state, init)  # capture leaves the state alone
    g.replay()
    torch.cuda.synchronize()
    e.device_status()
    assert torch.equal(e.state, eager_state)
    got = e.results(bg, 1.8)
    assert [r.energy for r in got] == [r.energy for r in eager]
    assert [r.n_p_plain for r in got] == [r.n_p_plain for r in eager]


def test_plan_must_match_ensemble(axs):
    from axion_strings_adaptive_gb300 import _lib as L
    bg = axs.Background.expanding(2.0, 1.0)
    e = _ensemble(axs, DIMS[:2], torch.float32)
    stale = L.EnsemblePlan.from_buffer_copy(bytes(e.plan))
    e.init(2, 5)
    with pytest.raises(L.AxsError):
        L.call("axs_ensemble_rk4_advance", C.byref(e.c), C.byref(stale), C.byref(bg.to_c()), 1.0, 0.0, 0.1, 1,
               torch.cuda.current_stream().cuda_stream)
    e.advance(bg, 1.0, 0.0, 0.1, 1)
    e.device_status()
