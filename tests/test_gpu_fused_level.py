"""The one-pass fused level step (level_fused.cuh) against the two-sweep step,
and the FP32 level step against the CPU oracle's FP32 and FP64 builds.

The fused step and the two sweeps evaluate the same per-site arithmetic, so the
state they leave (valid cells, periodic padding and its corners) must agree bit
for bit, whatever the step count (an odd count runs its first step as the two
sweeps, then fused pairs) and whatever the tile row (the first and last tile rows load their y
halo in wrapped pieces)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FUSED = ("f32 fused 32x16 ring6", "f32 fused 32x16 ring7", "f32 fused 32x16 ring6 t640",
         "f32 fused 32x16 ring7 t640")


def _config_id(lv, name):
    ids = [cid for cid, n in lv.tile_configs() if n == name]
    assert ids, f"tiling {name} not compiled"
    return ids[0]


def _state(shape, seed):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((4, nz, ny, nx))
    v[:2] += 2.0  # |psi| away from 0, Pi of order 1
    return torch.from_numpy(v).float()


def _run(axs, shape, cfg_name, v, steps, bg, dt=0.1):
    lv = axs.PeriodicLevel(shape, 0.5, dtype=torch.float32)
    if cfg_name is not None:
        lv.tile_config = _config_id(lv, cfg_name)
    lv.set_state(v.cuda())
    lv.advance(bg, 1.0, 0.0, dt, steps)
    lv.device_status()
    torch.cuda.synchronize()
    return lv


@pytest.mark.parametrize("shape", [(64, 64, 64), (96, 48, 40), (32, 16, 5), (64, 32, 3), (128, 80, 17), (32, 32, 1)])
@pytest.mark.parametrize("steps", [1, 2, 5])
def test_fused_step_is_bit_identical_to_two_sweeps(axs, shape, steps):
    v = _state(shape, sum(shape) + steps)
    bg = axs.Background.expanding(1.5, 1.0, lambda0=2.0)  # matter era: curvature term and lambda(tau) both live
    ref = _run(axs, shape, "f32 v2 64x8 ring8", v, steps, bg)
    for name in FUSED:
        got = _run(axs, shape, name, v, steps, bg)
        # the whole padded state: valid cells, periodic columns and rows, corners
        assert torch.equal(got.state, ref.state), (name, shape, steps)


def test_fused_step_keeps_padding_and_corners_current(axs):
    shape = (64, 48, 12)
    lv = _run(axs, shape, FUSED[0], _state(shape, 7), 3, axs.Background.flat(1.0), dt=0.05)
    st = lv.state.cpu().numpy()
    val = lv.get_state().cpu().numpy()
    ox, oy, nx, ny = lv.layout.x_offset, lv.layout.y_offset, lv.nx, lv.ny
    # padded rows oy-2 .. oy+ny+1 and columns ox-8 .. ox+nx+7 hold the periodic extension
    ys = (np.arange(-2, ny + 2) % ny)
    xs = (np.arange(-8, nx + 8) % nx)
    ext = val[:, :, ys][:, :, :, xs]
    np.testing.assert_array_equal(st[:, :, oy - 2:oy + ny + 2, ox - 8:ox + nx + 8], ext)


def test_unsupported_extent_falls_back_to_two_sweeps(axs):
    shape = (48, 20, 9)  # nx, ny not multiples of the fused tile
    v = _state(shape, 3)
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    ref = _run(axs, shape, "f32 v2 64x8 ring8", v, 4, bg)
    got = _run(axs, shape, FUSED[0], v, 4, bg)
    assert torch.equal(got.state, ref.state)


def _rel_max(a, b):
    return max(np.abs(a[c] - b[c]).max() / max(np.abs(b[c]).max(), 1e-300) for c in range(a.shape[0]))


def test_fp32_step_vs_oracle_fp32_and_fp64_builds(axs, orc):
    """The plain configuration (64^3, dx 0.5, dt 0.1, 100 steps, RD, c0 = 1,
    lambda0 = 2) in FP32 against the oracle's FP32 build (the reference's
    FLOAT build: stage-by-stage RK4 in float) and its FP64 build. The GPU path
    differs from the FLOAT build in arithmetic order (the stencil as
    differences from the centre, the step as increments rounded once per step),
    so the test bounds its distance to the FP64 result by the FLOAT build's own
    (max-norm per component relative to the component's maximum, worst
    component) and by 1e-5, and its distance to the FLOAT build by the sum of
    the two."""
    n, dx, dt, steps = 64, 0.5, 0.1, 100
    v = orc.fourier_ic_state(n, orc.strict_cutoff(n / 4), seed=1234)
    bgo = orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0)
    ref64 = orc.to_fab(v, 2)
    orc.rk4_advance(ref64, 2, dx, bgo, 1.0, 0.0, dt, steps)
    ref64 = orc.from_fab(ref64, 2)
    v32 = v.astype(np.float32)
    ref32 = orc.to_fab(v32, 2)  # float32 arrays run the oracle's FP32 build
    orc.rk4_advance(ref32, 2, dx, bgo, 1.0, 0.0, dt, steps)
    ref32 = orc.from_fab(ref32, 2).astype(np.float64)
    e_float_build = _rel_max(ref32, ref64)
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    for name in ("f32 v2 64x8 ring8",) + FUSED:
        lv = axs.PeriodicLevel(n, dx, dtype=torch.float32)
        lv.tile_config = _config_id(lv, name)
        lv.set_state(torch.from_numpy(v32).cuda())
        lv.advance(bg, 1.0, 0.0, dt, steps)
        lv.device_status()
        got = lv.get_state().double().cpu().numpy()
        e_gpu = _rel_max(got, ref64)
        assert e_gpu <= e_float_build and e_gpu < 1e-5, (name, e_gpu, e_float_build)
        assert _rel_max(got, ref32) <= e_gpu + e_float_build


@pytest.mark.parametrize("cfg", [None, "f32 v2 32x8 ring8 l2", "f32 fused 32x16 ring6 t640"])
@pytest.mark.parametrize("shape", [(64, 64, 64), (96, 48, 40), (32, 16, 5)])
def test_step_to_equals_an_in_place_step(axs, cfg, shape):
    """axs_level_rk4_step_to writes the in-place step's whole padded state into
    another buffer and leaves the level's state as it was."""
    v = _state(shape, 3 + sum(shape))
    bg = axs.Background.expanding(1.5, 1.0, lambda0=2.0)
    ref = _run(axs, shape, cfg, v, 1, bg)
    lv = axs.PeriodicLevel(shape, 0.5, dtype=torch.float32)
    if cfg is not None:
        lv.tile_config = _config_id(lv, cfg)
    lv.set_state(v.cuda())
    before = lv.state.clone()
    dst = torch.zeros_like(lv.state)
    lv.step_to(dst, bg, 1.0, 0.0, 0.1)
    lv.device_status()
    torch.cuda.synchronize()
    assert torch.equal(lv.state, before)
    assert torch.equal(dst, ref.state)
    old = lv.swap_state(dst)
    assert torch.equal(old, before) and lv.state.data_ptr() == dst.data_ptr()
    lv.advance(bg, 1.0, 0.1, 0.1, 1)  # the swapped-in buffer steps like any state
    ref.advance(bg, 1.0, 0.1, 0.1, 1)
    torch.cuda.synchronize()
    assert torch.equal(lv.state, ref.state)


def test_step_to_fp64(axs):
    shape = (48, 40, 24)
    rng = np.random.default_rng(5)
    v = torch.from_numpy(rng.standard_normal((4, shape[2], shape[1], shape[0])) + 1.5)
    bg = axs.Background.flat(1.0)
    a = axs.PeriodicLevel(shape, 0.5, dtype=torch.float64)
    a.set_state(v.cuda())
    b = axs.PeriodicLevel(shape, 0.5, dtype=torch.float64)
    b.set_state(v.cuda())
    dst = torch.zeros_like(b.state)
    a.advance(bg, 1.0, 0.0, 0.05, 1)
    b.step_to(dst, bg, 1.0, 0.0, 0.05)
    torch.cuda.synchronize()
    assert torch.equal(dst, a.state)


@pytest.mark.parametrize("shape", [(64, 64, 64), (96, 48, 40), (48, 40, 8)])
@pytest.mark.parametrize("steps", [1, 2, 3])
def test_compensated_step_is_bit_identical_across_tilings(axs, shape, steps):
    """AXS_LEVEL_COMPENSATED_FP32: the fused step (the default tiling) and the
    two sweeps it falls back to (single and odd steps, extents it does not take,
    other tilings) evaluate the same compensated arithmetic."""
    v = _state(shape, 11 + sum(shape) + steps)
    bg = axs.Background.expanding(1.5, 1.0, lambda0=2.0)
    out = []
    for name in ("f32 fused 32x16 ring6 t640", "f32 v2 32x8 ring8 l2", "f32 v2 64x8 ring8"):
        lv = axs.PeriodicLevel(shape, 0.5, dtype=torch.float32)
        lv.tile_config = _config_id(lv, name)
        lv.compensated = True
        lv.set_state(v.cuda())
        lv.advance(bg, 1.0, 0.0, 0.1, steps)
        lv.device_status()
        out.append(lv.state.clone())
    torch.cuda.synchronize()
    assert torch.equal(out[0], out[1]) and torch.equal(out[0], out[2])
    plain = _run(axs, shape, "f32 fused 32x16 ring6 t640", v, steps, bg)
    assert not torch.equal(plain.state, out[0])  # the compensation changes the bits


def test_compensated_fp32_step_vs_oracle_fp64(axs, orc):
    """The plain configuration (64^3, 100 steps) in compensated FP32 against the
    oracle's FP64 build: within the FP32 bound the plain step meets (max-norm
    per component relative to its maximum, worst component). The compensation
    removes a bias shared by every site, which shows in sums over a large box
    (the benchmark's 512^3 precision report), not in a pointwise norm at 64^3."""
    n, dx, dt, steps = 64, 0.5, 0.1, 100
    v = orc.fourier_ic_state(n, orc.strict_cutoff(n / 4), seed=1234)
    bgo = orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0)
    ref64 = orc.to_fab(v, 2)
    orc.rk4_advance(ref64, 2, dx, bgo, 1.0, 0.0, dt, steps)
    ref64 = orc.from_fab(ref64, 2)
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lv = axs.PeriodicLevel(n, dx, dtype=torch.float32)
    lv.compensated = True
    lv.set_state(torch.from_numpy(v.astype(np.float32)).cuda())
    lv.advance(bg, 1.0, 0.0, dt, steps)
    lv.device_status()
    assert _rel_max(lv.get_state().double().cpu().numpy(), ref64) < 1e-5
