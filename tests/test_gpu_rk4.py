"""GPU parity of the RHS and the RK4 time step against the CPU oracle and the
reference-generated golden fixtures (all calls go through the C ABI)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _to_dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def _fab_from_valid(A, valid, ng, dtype):
    c, nz, ny, nx = valid.shape
    t = A.new_fab((nx, ny, nz), ng, dtype=dtype, ncomp=c)
    A.valid(t, ng).copy_(_to_dev(valid, dtype))
    A.fill_periodic_ghosts(t, ng)
    return t


def _rel_max(a, b):
    """max over planes of max|a-b| / max|b| (per component)."""
    out = 0.0
    for c in range(a.shape[0]):
        scale = max(np.abs(b[c]).max(), 1e-300)
        out = max(out, np.abs(a[c] - b[c]).max() / scale)
    return out


@pytest.mark.parametrize("box", ["rand", "ic"])
def test_eval_rhs_f64_bit_exact_vs_reference(axs, golden, box):
    g = golden("fields_f64.npz")
    dx, kappa, lam, R2 = g["params"][:4]
    soln = _fab_from_valid(axs, g[f"{box}_state"], 2, torch.float64)
    c, nz, ny, nx = g[f"{box}_state"].shape
    rhs = axs.new_fab((nx, ny, nz), 0, dtype=torch.float64)
    coeffs = axs._lib.RhsCoeffs(kappa, lam, R2)
    axs.eval_rhs(soln, rhs, 2, 0, dx, coeffs)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(rhs.cpu().numpy(), g[f"{box}_rhs"])


@pytest.mark.parametrize("box", ["rand", "ic"])
def test_eval_rhs_f32_vs_reference_float_build(axs, golden, box):
    g = golden("fields_f32.npz")
    dx, kappa, lam, R2 = g["params"][:4]
    soln = _fab_from_valid(axs, g[f"{box}_state"], 2, torch.float32)
    c, nz, ny, nx = g[f"{box}_state"].shape
    rhs = axs.new_fab((nx, ny, nz), 1, dtype=torch.float32)
    axs.eval_rhs(soln, rhs, 2, 1, dx, axs._lib.RhsCoeffs(kappa, lam, R2))
    got = axs.valid(rhs, 1).cpu().numpy()
    ref = g[f"{box}_rhs"]
    np.testing.assert_array_equal(got[:2], ref[:2])  # rhs_psi = Pi exactly
    # FP32 arithmetic order differs from the FLOAT build's double-weight diff2: a few ulp of the stencil scale
    scale = np.abs(g[f"{box}_state"][:2]).max() * 16 / dx ** 2 * 3
    assert np.abs(got[2:] - ref[2:]).max() <= 4e-6 * scale


def test_fill_lincomb_combine(axs, orc):
    rng = np.random.default_rng(5)
    v = rng.standard_normal((4, 6, 7, 8))
    t = _fab_from_valid(axs, v, 2, torch.float64)
    f = orc.to_fab(v, 2)
    np.testing.assert_array_equal(t.cpu().numpy(), f)
    x = _fab_from_valid(axs, rng.standard_normal((4, 6, 7, 8)), 2, torch.float64)
    y = _fab_from_valid(axs, rng.standard_normal((4, 6, 7, 8)), 2, torch.float64)
    d = torch.zeros_like(x)
    axs.lincomb(d, x, 0.37, y, 2)
    xv, yv = axs.valid(x, 2).cpu().numpy(), axs.valid(y, 2).cpu().numpy()
    np.testing.assert_array_equal(axs.valid(d, 2).cpu().numpy(), xv + 0.37 * yv)  # no contraction
    ks = [_fab_from_valid(axs, rng.standard_normal((4, 6, 7, 8)), 2, torch.float64) for _ in range(4)]
    axs.rk4_combine(d, x, *ks, 2, 0.1)
    V = [axs.valid(k, 2).cpu().numpy() for k in ks]
    ref = axs.valid(x, 2).cpu().numpy() + (0.1 / 6) * (V[0] + 2 * V[1] + 2 * V[2] + V[3])
    np.testing.assert_array_equal(axs.valid(d, 2).cpu().numpy(), ref)


def _stagewise_rk4(axs, state_valid, dx, bg, tau_i, t0, dt, nsteps):
    """The drop-in path: per-stage specific_eval_rhs + LinComb, as GRTeclyn drives it."""
    ng = 2
    c, nz, ny, nx = state_valid.shape
    u = _fab_from_valid(axs, state_valid, ng, torch.float64)
    uold, us = torch.zeros_like(u), torch.zeros_like(u)
    ks = [torch.zeros_like(u) for _ in range(4)]
    lvl = axs.AxionStringsLevel((nx, ny, nz), dx, bg, tau_i=tau_i, dtype=torch.float64)
    t = t0
    for _ in range(nsteps):
        uold.copy_(u)
        for s, (ts, cs) in enumerate(((t, 0.5 * dt), (t + 0.5 * dt, 0.5 * dt), (t + 0.5 * dt, dt), (t + dt, None))):
            src = uold if s == 0 else us
            axs.fill_periodic_ghosts(src, ng)
            lvl.specific_eval_rhs(src, ks[s], ts, ng_soln=ng, ng_rhs=ng)
            if cs is not None:
                axs.lincomb(us, uold, cs, ks[s], ng)
        axs.rk4_combine(u, uold, *ks, ng, dt)
        t += dt
    return axs.valid(u, ng).cpu().numpy()


def test_stagewise_rk4_matches_oracle(axs, orc):
    rng = np.random.default_rng(11)
    v = rng.standard_normal((4, 10, 12, 16)) * np.array([1, 1, .3, .3])[:, None, None, None]
    dx, dt, n = 0.5, 0.1, 6
    bgo = orc.background(a_inv=1.5, c0=1.0, lambda_scale=2.0)
    fab = orc.to_fab(v, 2)
    orc.rk4_advance(fab, 2, dx, bgo, 1.0, 0.0, dt, n)
    ref = orc.from_fab(fab, 2)
    got = _stagewise_rk4(axs, v, dx, axs.Background.expanding(1.5, 1.0, lambda0=2.0), 1.0, 0.0, dt, n)
    # FP64 RHS and stage combinations evaluate the same expressions with the same
    # rounding as the CPU restatement: bit-exact
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("shape", [(16, 12, 10), (32, 20, 7), (48, 33, 16), (8, 4, 5), (4, 2, 3)])
def test_fused_rk4_f64_matches_oracle(axs, orc, shape):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz)
    v = rng.standard_normal((4, nz, ny, nx)) * np.array([1, 1, .3, .3])[:, None, None, None]
    dx, dt, n = 0.5, 0.1, 12
    # matter domination (a_inv = 1.5): nonzero curvature term, time-dependent lambda -> stage times matter
    bgo = orc.background(a_inv=1.5, c0=1.0, lambda_scale=2.0)
    fab = orc.to_fab(v, 2)
    orc.rk4_advance(fab, 2, dx, bgo, 1.0, 0.0, dt, n)
    ref = orc.from_fab(fab, 2)
    lv = axs.PeriodicLevel((nx, ny, nz), dx, dtype=torch.float64)
    lv.set_state(_to_dev(v))
    lv.advance(axs.Background.expanding(1.5, 1.0, lambda0=2.0), 1.0, 0.0, dt, n)
    lv.device_status()
    got = lv.get_state().cpu().numpy()
    assert _rel_max(got, ref) < 1e-12


def test_fused_rk4_config_plain_64cubed_100_steps(axs, orc):
    """64^3, dx=0.5, dt=0.1, 100 steps, RD (a_inv=2), fat strings (c0=1), lambda0=2, FP64:
    fields within 1e-10 relative of the oracle."""
    n, dx, dt, steps = 64, 0.5, 0.1, 100
    v = orc.fourier_ic_state(n, orc.strict_cutoff(n / 4), seed=1234)
    bgo = orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0)
    fab = orc.to_fab(v, 2)
    orc.rk4_advance(fab, 2, dx, bgo, 1.0, 0.0, dt, steps)
    ref = orc.from_fab(fab, 2)
    lv = axs.PeriodicLevel(n, dx, dtype=torch.float64)
    lv.set_state(_to_dev(v))
    lv.advance(axs.Background.expanding(2.0, 1.0, lambda0=2.0), 1.0, 0.0, dt, steps)
    lv.device_status()
    got = lv.get_state().cpu().numpy()
    assert _rel_max(got, ref) < 1e-10


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-13), (torch.float32, 2e-5)])
def test_homogeneous_solution_is_exact(axs, dtype, tol):
    """psi = R(tau), Pi = R'(tau) solves the full EOM (test_background.cpp:69-89);
    in radiation domination R = tau is linear, which RK4 integrates exactly."""
    n, dx, dt, steps = 16, 0.5, 0.1, 40
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    v = torch.zeros((4, n, n, n), dtype=torch.float64)
    v[0] = bg.R(1.0)
    v[2] = bg.R_prime(1.0)
    lv = axs.PeriodicLevel(n, dx, dtype=dtype)
    lv.set_state(v.cuda())
    lv.advance(bg, 1.0, 0.0, dt, steps)
    s = lv.get_state().double().cpu()
    tau_f = 1.0 + steps * dt
    assert torch.allclose(s[0], torch.full_like(s[0], bg.R(tau_f)), rtol=tol, atol=0)
    assert torch.allclose(s[2], torch.full_like(s[2], bg.R_prime(tau_f)), rtol=tol, atol=tol)
    assert float(s[1].abs().max()) == 0.0 and float(s[3].abs().max()) == 0.0


def _check_padding(lv, val):
    """The 8 columns either side in x (whole 32-byte sectors; the stencils read 4)
    and 2 rows either side in y hold periodic copies (nx >= 8)."""
    st = lv.state.cpu().numpy()
    ox, oy, nx, ny = lv.layout.x_offset, lv.layout.y_offset, lv.nx, lv.ny
    rows = st[:, :, oy:oy + ny]
    np.testing.assert_array_equal(rows[..., ox - 8:ox], val[..., nx - 8:nx])
    np.testing.assert_array_equal(rows[..., ox + nx:ox + nx + 8], val[..., :8])
    np.testing.assert_array_equal(st[:, :, oy - 2:oy, ox:ox + nx], val[:, :, ny - 2:ny, :])
    np.testing.assert_array_equal(st[:, :, oy + ny:oy + ny + 2, ox:ox + nx], val[:, :, :2, :])


def test_level_fab_round_trip(axs):
    rng = np.random.default_rng(3)
    v = rng.standard_normal((4, 9, 10, 12))
    t = _fab_from_valid(axs, v, 3, torch.float64)
    lv = axs.PeriodicLevel((12, 10, 9), 0.5, dtype=torch.float64)
    lv.import_fab(t, 3)
    np.testing.assert_array_equal(lv.get_state().cpu().numpy(), v)
    out = axs.new_fab((12, 10, 9), 1, dtype=torch.float64)
    lv.export_fab(out, 1)
    np.testing.assert_array_equal(axs.valid(out, 1).cpu().numpy(), v)
    # padding holds periodic copies
    _check_padding(lv, v)


def test_fused_rk4_keeps_padding_current(axs):
    rng = np.random.default_rng(8)
    v = rng.standard_normal((4, 8, 6, 8)) * 0.5
    lv = axs.PeriodicLevel((8, 6, 8), 0.5, dtype=torch.float64)
    lv.set_state(_to_dev(v))
    lv.advance(axs.Background.flat(1.0), 0.0, 0.0, 0.05, 3)
    _check_padding(lv, lv.get_state().cpu().numpy())


def test_fused_rk4_f64_512cubed_matches_oracle(axs, orc):
    """The precision workload's grid in FP64 (512^3, dx 0.5, Moore c0 = 2,
    lambda0 = 2, RD, Fourier IC |n| < N/8), 2 steps, against the oracle's
    stage-by-stage RK4: element offsets past 32 bits on real 3-D data. The
    oracle holds about 40 GB on the host."""
    import os
    if os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES") < 96 * 2 ** 30:
        pytest.skip("the 512^3 FP64 oracle needs about 40 GB of host memory")
    from axion_strings_adaptive_gb300 import ic
    n, dx, dt, steps = 512, 0.5, 0.1, 2
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=31, dtype=torch.float64, device="cuda")
    lv = axs.PeriodicLevel(n, dx, dtype=torch.float64, pierced_capacity=1024)
    lv.set_state(s0)
    lv.advance(axs.Background.expanding(2.0, 2.0, lambda0=2.0), 1.0, 0.0, dt, steps)
    lv.device_status()
    got = lv.get_state().cpu().numpy()
    v = s0.cpu().numpy()
    del lv, s0
    torch.cuda.empty_cache()
    fab = orc.to_fab(v, 2)
    del v
    orc.rk4_advance(fab, 2, dx, orc.background(a_inv=2.0, c0=2.0, lambda_scale=2.0), 1.0, 0.0, dt, steps)
    ref = orc.from_fab(fab, 2)
    del fab
    assert _rel_max(got, ref) < 1e-12


@pytest.mark.parametrize("shape", [(64, 16, 40), (32, 8, 5), (96, 24, 70)])
def test_eval_rhs_f32_wide_staging_equals_cell_staging(axs, shape):
    """FP32 drop-in RHS: FABs with ng = 2 and tile-multiple extents stage their
    rows in 16-byte pieces, others cell by cell; same arithmetic, same bits."""
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + nz)
    v = torch.from_numpy(rng.standard_normal((4, nz, ny, nx)) + 1.0).float().cuda()
    c = axs.Background.expanding(2.0, 2.0, lambda0=2.0).rhs_coeffs(1.7)
    out = []
    for ng in (2, 3):
        s = axs.new_fab((nx, ny, nz), ng, dtype=torch.float32)
        axs.valid(s, ng).copy_(v)
        axs.fill_periodic_ghosts(s, ng)
        r = axs.new_fab((nx, ny, nz), 0, dtype=torch.float32)
        axs.eval_rhs(s, r, ng, 0, 0.5, c)
        out.append(axs.valid(r, 0).clone())
    torch.cuda.synchronize()
    assert torch.equal(out[0], out[1])
