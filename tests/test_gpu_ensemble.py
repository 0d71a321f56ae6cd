"""Ensemble (batching) path through the C ABI: boxes of uneven sizes packed in
one arena and advanced together (one persistent launch per sweep, or one fused
launch per step) evolve bit for bit as the same boxes advanced one level at a
time, for every compiled tiling and z-chunk target and for even and odd step
counts; the fused step's padding equals a ghost fill; per-box diagnostics
equal the level diagnostics; a captured CUDA graph replays the eager run
exactly."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu

DIMS = [(32, 32, 32), (48, 40, 24), (64, 16, 36), (24, 28, 12), (16, 16, 8)]
# boxes the fused step takes: ny a multiple of 16, nx even (48 and 16 leave a partial tile column)
DIMS_FUSED = [(32, 32, 32), (48, 48, 24), (96, 16, 36), (16, 32, 12), (64, 16, 8)]


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


def _fused_id(e):
    ids = [cid for cid, name in e.tile_configs() if "fused" in name]
    assert len(ids) == 1
    return ids[0]


@pytest.mark.parametrize("dims,steps", [(DIMS, 4), (DIMS_FUSED, 4), (DIMS_FUSED, 3)], ids=["odd", "fused", "fused-odd"])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_ensemble_matches_levels_bitwise_every_tiling(axs, dtype, dims, steps):
    from axion_strings_adaptive_gb300 import _lib as L
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    ref = [lv.get_state() for lv in _levels(axs, dims, dtype, bg, steps)]
    e = _ensemble(axs, dims, dtype)
    init = e.state.clone()
    ran = []
    for cid, name in [(0, "default")] + e.tile_configs():
        for zc in (0, 3, 7):
            e.state.copy_(init)
            try:
                e.init(cid, zc)
            except L.AxsError as err:
                # only the fused tiling refuses boxes, and only boxes it cannot take
                assert err.status == L.AXS_ERR_UNSUPPORTED and "fused" in name and dims is DIMS, (name, err)
                break
            e.advance(bg, 1.0, 0.0, 0.1, steps)
            e.device_status()
            for b in range(len(dims)):
                assert torch.equal(e.get_box(b), ref[b]), (name, zc, b)
            ran.append(name)
    if dtype == torch.float32 and dims is DIMS_FUSED:
        assert any("fused" in n for n in ran)


@pytest.mark.parametrize("steps", [2, 5])
def test_fused_ensemble_padding_equals_ghost_fill(axs, steps):
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    e = _ensemble(axs, DIMS_FUSED, torch.float32)
    e.init(_fused_id(e), 0)
    e.advance(bg, 1.0, 0.0, 0.1, steps)
    e.device_status()
    after = e.state.clone()
    e.fill_ghosts()
    assert torch.equal(e.state, after)


@pytest.mark.parametrize("steps", [8, 7])
def test_fused_graph_replay_equals_eager(axs, steps):
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    e = _ensemble(axs, DIMS_FUSED, torch.float32)
    e.init(_fused_id(e), 0)
    init = e.state.clone()
    e.advance(bg, 1.0, 0.0, 0.1, steps)
    eager_state = e.state.clone()
    e.state.copy_(init)
    g = e.capture(bg, 1.0, 0.0, 0.1, steps, diagnostics=False)
    g.replay()
    torch.cuda.synchronize()
    e.device_status()
    assert torch.equal(e.state, eager_state)


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
