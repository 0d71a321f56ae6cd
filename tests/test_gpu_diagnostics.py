"""GPU parity of the fused diagnostics pass (string finder, energy sums,
velocities) and the small device entry points, through the C ABI, against the
reference-generated golden fixtures and the CPU oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def _run_diag(axs, fab_t, ng, params, mask=None, capacity=None):
    L = axs._lib
    f = axs.fab(fab_t, ng)
    ncell = f.nx * f.ny * f.nz
    scratch = torch.zeros(axs.level.scratch_bytes(f.nx, f.ny, f.nz), dtype=torch.uint8, device="cuda")
    res = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device="cuda")
    cap = 3 * ncell if capacity is None else capacity
    lst = torch.full((max(cap, 1),), -1, dtype=torch.int64, device="cuda")
    m = None if mask is None else _dev(mask.astype(np.uint8)).reshape(-1)
    L.call("axs_diagnostics", C.byref(f), C.byref(params), None if m is None else m.data_ptr(), res.data_ptr(),
           lst.data_ptr(), cap, scratch.data_ptr(), scratch.numel(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    r = L.DiagResult.from_buffer_copy(res.cpu().numpy().tobytes())
    return r, lst[: min(r.n_listed, cap)].cpu().numpy()


def _params(axs, g, scheme, boundary, want=(1, 1, 1), prec="f64"):
    dx, kappa, lam, R2, R, RpR, m_r = g["params"]
    if prec == "f32":  # the FLOAT build receives R, lambda, R'/R, m_r as amrex::Real (EnergyKernel.hpp:107-109)
        dx, lam, R, RpR, m_r = (float(np.float32(x)) for x in (dx, lam, R, RpR, m_r))
    return axs._lib.DiagParams(dx, R, lam, RpR, m_r, scheme, 0.8, boundary, *want)


def _pierced_from_windings(w):
    nz, ny, nx, _ = w.shape
    cells = np.arange(nx * ny * nz).reshape(nz, ny, nx)
    out = []
    for pl in range(3):
        out.append(4 * cells[w[..., pl] != 0] + pl)
    return np.sort(np.concatenate(out))


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["rand", "ic"])
@pytest.mark.parametrize("boundary", ["ghosts", "periodic"])
def test_diagnostics_vs_reference(axs, golden, prec, box, boundary):
    g = golden(f"fields_{prec}.npz")
    dt = torch.float64 if prec == "f64" else torch.float32
    st = g[f"{box}_state"]
    c, nz, ny, nx = st.shape
    ng = 2 if boundary == "ghosts" else 0
    t = axs.new_fab((nx, ny, nz), ng, dtype=dt)
    axs.valid(t, ng).copy_(_dev(st, dt))
    if ng:
        axs.fill_periodic_ghosts(t, ng)
    bmode = axs._lib.BOUNDARY_GHOSTS if ng else axs._lib.BOUNDARY_PERIODIC
    for scheme in range(3):
        r, lst = _run_diag(axs, t, ng, _params(axs, g, scheme, bmode, prec=prec))
        assert r.status == 0 and r.n_near_tie == 0
        assert (r.n_p_plain, r.n_p_weighted) == tuple(g[f"{box}_counts"])
        np.testing.assert_array_equal(np.sort(lst), _pierced_from_windings(g[f"{box}_windings"]))
        np.testing.assert_allclose(list(r.energy_sums), g[f"{box}_energy_sums"][scheme], rtol=1e-12, atol=1e-300)
        vs, vc = g[f"{box}_velocity"]
        if prec == "f64":  # the FLOAT build recomputes windings with float atan2 (VelocityKernel.hpp:66-69)
            assert r.vel_count == int(vc)
            assert r.vel_sum == pytest.approx(vs, rel=1e-12)
    # coverage mask
    r, _ = _run_diag(axs, t, ng, _params(axs, g, 1, bmode, prec=prec), mask=g[f"{box}_mask"])
    assert (r.n_p_plain, r.n_p_weighted) == tuple(g[f"{box}_counts_masked"])
    np.testing.assert_allclose(list(r.energy_sums), g[f"{box}_energy_sums_masked"], rtol=1e-12, atol=1e-300)


def test_velocity_matches_oracle_f32(axs, orc, golden):
    g = golden("fields_f32.npz")
    dx, kappa, lam, R2, R, RpR, m_r = (float(np.float32(x)) for x in g["params"])
    st = g["ic_state"]
    fab = orc.to_fab(st, 2)
    # oracle with the GPU's phase precision (double atan2) for the pierced set
    from oracle.oracle import velocity
    vs_native, vc_native = velocity(fab, 2, R, RpR, m_r)
    t = axs.new_fab(st.shape[1:][::-1], 2, dtype=torch.float32)
    axs.valid(t, 2).copy_(_dev(st))
    axs.fill_periodic_ghosts(t, 2)
    r, _ = _run_diag(axs, t, 2, _params(axs, g, 1, axs._lib.BOUNDARY_GHOSTS, prec="f32"))
    # smooth field: float and double atan2 agree on every winding here
    assert r.vel_count == vc_native
    assert r.vel_sum == pytest.approx(vs_native, rel=1e-12)


@pytest.mark.parametrize("box", ["rand", "ic"])
def test_fp32_velocity_matches_float_build_fixture(axs, orc, golden, box):
    """FP32 velocity against the reference's own FLOAT build. The FLOAT build
    recomputes the windings it sums over with float atan2
    (VelocityKernel.hpp:66-69); the GPU sums over the string finder's pierced
    set, which uses double atan2 (StringFinder.hpp:49-53) in both precisions,
    so that counts, list and velocities refer to the same plaquettes. The two
    sets differ only where a float phase difference lands on the other side
    of +-pi. The test counts that difference on the CPU (oracle, double atan2,
    against the fixture's count); on these boxes it is zero, and the velocity
    count and sum then equal the FLOAT build's."""
    g = golden("fields_f32.npz")
    st = g[f"{box}_state"]
    plain_double, _ = orc.count_plaquettes(orc.to_fab(st, 2), 2)
    vs_f, vc_f = g[f"{box}_velocity"]
    set_difference = int(vc_f) // 4 - plain_double  # plaquettes pierced only under float atan2 (net)
    t = axs.new_fab(st.shape[1:][::-1], 2, dtype=torch.float32)
    axs.valid(t, 2).copy_(_dev(st))
    axs.fill_periodic_ghosts(t, 2)
    r, _ = _run_diag(axs, t, 2, _params(axs, g, 1, axs._lib.BOUNDARY_GHOSTS, prec="f32"))
    assert r.vel_count == 4 * r.n_p_plain == 4 * plain_double
    assert set_difference == 0
    assert r.vel_count == int(vc_f)
    assert r.vel_sum == pytest.approx(vs_f, rel=1e-12)


def test_level_diagnostics_matches_oracle(axs, orc):
    n, dx = 24, 0.5
    v = orc.fourier_ic_state(n, 5.0, seed=99)
    v[2:] = 0.3 * np.random.default_rng(1).standard_normal((2, n, n, n))
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    bgo = orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0)
    tau = 1.7
    lvl = axs.PeriodicLevel(n, dx, dtype=torch.float64)
    lvl.set_state(_dev(v))
    d = lvl.diagnostics(bg, tau)
    ref = orc.level_diagnostics(v, dx, bgo, tau)
    assert (d.n_p_plain, d.n_p_weighted) == (ref.n_p_plain, ref.n_p_weighted)
    np.testing.assert_allclose(d.energy_sums, ref.energy_sums, rtol=1e-12)
    assert d.xi_plain == pytest.approx(ref.xi_plain, rel=1e-14)
    assert d.vel_count == ref.vel_count
    assert d.mean_gamma_sq_v_sq == pytest.approx(ref.mean_gamma_sq_v_sq, rel=1e-12)
    assert d.energy["rho_tot_unscreened"] == pytest.approx(ref.energy[0], rel=1e-12)
    assert d.energy["rho_tot_screened"] == pytest.approx(ref.energy[1], rel=1e-12)


def test_pierced_list_capacity(axs, golden):
    g = golden("fields_f64.npz")
    st = g["rand_state"]
    c, nz, ny, nx = st.shape
    t = axs.new_fab((nx, ny, nz), 0, dtype=torch.float64)
    t.copy_(_dev(st))
    r, lst = _run_diag(axs, t, 0, _params(axs, g, 1, axs._lib.BOUNDARY_PERIODIC), capacity=10)
    assert r.status == axs._lib.AXS_ERR_CAPACITY
    assert r.n_listed == 10 and r.n_p_plain == g["rand_counts"][0]  # counts stay exact
    full = set(_pierced_from_windings(g["rand_windings"]).tolist())
    assert set(lst.tolist()) <= full


def test_winding_kats_on_device(axs, golden):
    g = golden("kats.npz")
    th = _dev(g["winding_theta"]).contiguous()
    w = torch.zeros(th.shape[0], dtype=torch.int32, device="cuda")
    axs._lib.call("axs_plaquette_winding_batch", th.data_ptr(), th.shape[0], w.data_ptr(),
                  torch.cuda.current_stream().cuda_stream)
    np.testing.assert_array_equal(w.cpu().numpy(), g["winding_w"])


def test_fourier_spectrum_and_ic(axs, orc, golden):
    from axion_strings_adaptive_gb300 import ic
    for (nx, ny, nz, kmax, seed, comp) in ((16, 16, 16, 4.0, 4242, 0), (12, 10, 8, 3.2, 99, 1),
                                          (32, 32, 32, ic.strict_cutoff(8), 7, 1)):
        ref = orc.fourier_spectrum(nx, ny, nz, kmax, seed, comp)
        spec = torch.zeros((nz, ny, nx // 2 + 1, 2), dtype=torch.float64, device="cuda")
        axs._lib.call("axs_fourier_spectrum", spec.data_ptr(), nx, ny, nz, kmax, seed, comp,
                      torch.cuda.current_stream().cuda_stream)
        got = spec.cpu().numpy()
        np.testing.assert_allclose(got[..., 0] + 1j * got[..., 1], ref, rtol=0, atol=5e-15)
    gf = golden("fourier_ic.npz")
    nx, ny, nz, kmax, seed, comp = gf["a_args"]
    f = ic.fourier_component((int(nx), int(ny), int(nz)), kmax, int(seed), int(comp))
    np.testing.assert_allclose(f.cpu().numpy(), gf["a_field"], rtol=0, atol=1e-13)


def test_rejects_bad_arguments_without_launching(axs):
    L = axs._lib
    f = L.Fab(None, L.AXS_F64, 8, 8, 8, 2, 4, 12, 144, 1728)
    c = L.RhsCoeffs(0.0, 1.0, 1.0)
    assert L.lib().axs_eval_rhs(C.byref(f), C.byref(f), 0.5, C.byref(c), None) == L.AXS_ERR_INVALID_ARGUMENT
    t = axs.new_fab((8, 8, 8), 1, dtype=torch.float64)
    assert L.lib().axs_eval_rhs(C.byref(axs.fab(t, 1)), C.byref(axs.fab(t, 1)), 0.5, C.byref(c),
                                None) == L.AXS_ERR_INVALID_ARGUMENT  # needs 2 ghosts
    assert b"ghost" in L.lib().axs_last_error()


def test_per_cell_fp32_variant(axs):
    """per_cell_fp32 on FP32 fields: identical winding counts, pierced list and
    velocity count; energy sums within 2e-6 relative of the double per-cell pass."""
    from axion_strings_adaptive_gb300 import ic
    n = 64
    bg = axs.Background.expanding(2.0, 2.0, lambda0=2.0)
    lv = axs.PeriodicLevel(n, 0.5, dtype=torch.float32)
    lv.set_state(ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=5).float())
    lv.advance(bg, 1.0, 0.0, 0.1, 30)
    lv.device_status()
    ref = lv.diagnostics(bg, 4.0)
    fast = lv.diagnostics(bg, 4.0, per_cell_fp32=True)
    assert (fast.n_p_plain, fast.n_p_weighted, fast.vel_count) == (ref.n_p_plain, ref.n_p_weighted, ref.vel_count)
    assert torch.equal(torch.sort(fast.pierced)[0], torch.sort(ref.pierced)[0])
    np.testing.assert_allclose(fast.energy_sums, ref.energy_sums, rtol=2e-6)
    assert fast.mean_gamma_sq_v_sq == pytest.approx(ref.mean_gamma_sq_v_sq, rel=1e-5)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_exact_zeros_and_a_vacuum_corner_match_oracle(axs, orc, dtype):
    """Cells where psi is exactly zero (a core on a grid point: atan2(0, 0) = 0,
    the 1/|psi|^2 guards) and a block of the false vacuum psi = 0, Pi = 0."""
    n, dx = 16, 0.5
    v = orc.fourier_ic_state(n, 4.0, seed=5)
    v[2:] = 0.2 * np.random.default_rng(2).standard_normal((2, n, n, n))
    rng = np.random.default_rng(3)
    zs = rng.integers(0, n, size=(40, 3))
    v[0, zs[:, 0], zs[:, 1], zs[:, 2]] = 0.0
    v[1, zs[:, 0], zs[:, 1], zs[:, 2]] = 0.0
    v[:, :4, :4, :4] = 0.0
    if dtype == torch.float32:
        v = v.astype(np.float32).astype(np.float64)  # the same values on both sides
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    bgo = orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0)
    tau = 1.3
    lvl = axs.PeriodicLevel(n, dx, dtype=dtype)
    lvl.set_state(_dev(v).to(dtype))
    d = lvl.diagnostics(bg, tau)
    ref = orc.level_diagnostics(v, dx, bgo, tau)
    assert (d.n_p_plain, d.n_p_weighted) == (ref.n_p_plain, ref.n_p_weighted)
    assert np.all(np.isfinite(d.energy_sums))
    if dtype == torch.float64:
        np.testing.assert_allclose(d.energy_sums, ref.energy_sums, rtol=1e-12)
        assert d.vel_count == ref.vel_count


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["rand", "ic"])
@pytest.mark.parametrize("boundary", ["ghosts", "periodic"])
def test_string_finder_alone_vs_reference(axs, golden, prec, box, boundary):
    """The windings-only pass (the edge-code finder): the reference's counts and
    pierced set, with and without a coverage mask."""
    g = golden(f"fields_{prec}.npz")
    dt = torch.float64 if prec == "f64" else torch.float32
    st = g[f"{box}_state"]
    c, nz, ny, nx = st.shape
    ng = 2 if boundary == "ghosts" else 0
    t = axs.new_fab((nx, ny, nz), ng, dtype=dt)
    axs.valid(t, ng).copy_(_dev(st, dt))
    if ng:
        axs.fill_periodic_ghosts(t, ng)
    bmode = axs._lib.BOUNDARY_GHOSTS if ng else axs._lib.BOUNDARY_PERIODIC
    r, lst = _run_diag(axs, t, ng, _params(axs, g, 1, bmode, want=(0, 1, 0), prec=prec))
    assert r.status == 0 and r.n_near_tie == 0
    assert (r.n_p_plain, r.n_p_weighted) == tuple(g[f"{box}_counts"])
    assert list(r.energy_sums) == [0.0] * 14 and r.vel_count == 0
    np.testing.assert_array_equal(np.sort(lst), _pierced_from_windings(g[f"{box}_windings"]))
    r, _ = _run_diag(axs, t, ng, _params(axs, g, 1, bmode, want=(0, 1, 0), prec=prec), mask=g[f"{box}_mask"])
    assert (r.n_p_plain, r.n_p_weighted) == tuple(g[f"{box}_counts_masked"])


def _finder_cases(orc, n):
    rng = np.random.default_rng(11)
    v = orc.fourier_ic_state(n, 4.0, seed=8)
    v[2:] = 0.0
    yield "ic", v
    # exact zeros (atan2(0, 0)), a false-vacuum block and huge values: vertices outside float range
    w = v.copy()
    zs = rng.integers(0, n, size=(60, 3))
    w[:2, zs[:, 0], zs[:, 1], zs[:, 2]] = 0.0
    w[:2, :5, :3, :4] = 0.0
    w[:2, 7, 7, 7] = 1e31
    yield "zeros", w
    # phases pi apart on every x edge: every cell goes to the double path, with
    # near-ties counted
    u = np.zeros_like(v)
    x = np.arange(n)
    u[0] = np.where(x % 2 == 0, 1.0, -1.0)[None, None, :] * (1.0 + 0.1 * rng.random((n, n, n)))
    u[1] = np.where((x // 2) % 3 == 0, 0.0, 1e-9) * rng.standard_normal((n, n, n))
    yield "pi", u
    # random phases: many pierced plaquettes, many list flushes per block
    r = rng.standard_normal((4, n, n, n))
    r[2:] = 0.0
    yield "rand", r
    # phases on multiples of pi/4: vertices on the real axis (imaginary parts +0
    # and -0), edges exactly pi apart, tiny and zero magnitudes
    k = rng.integers(0, 8, size=(n, n, n))
    mag = rng.choice([0.5, 1.0, 2.0, 1e-20, 0.0], size=(n, n, n), p=[0.3, 0.3, 0.3, 0.05, 0.05])
    a = np.zeros_like(v)
    a[0] = mag * np.cos(k * np.pi / 4)
    a[1] = mag * np.sin(k * np.pi / 4)
    on_axis = k % 4 == 0
    a[1][on_axis] = np.where(rng.random(on_axis.sum()) < 0.5, 0.0, -0.0)
    a[0][k % 4 == 2] = 0.0
    yield "axes", a


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n", [24, 40])
def test_string_finder_alone_equals_fused_pass(axs, orc, dtype, n):
    """The windings-only finder (FP32: the phase-free finder; FP64: the
    edge-code finder) against the fused pass (itself pinned to the reference
    above): counts, near-ties and the pierced set, on fields that take the
    double fall-back (zeros, huge values, edges pi apart, phases on the real
    axis with signed zeros) and on a dense random field, at a size that leaves
    partial tiles."""
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    for name, v in _finder_cases(orc, n):
        lvl = axs.PeriodicLevel(n, 0.5, dtype=dtype, pierced_capacity=3 * n ** 3)
        lvl.set_state(_dev(v).to(dtype))
        full = lvl.diagnostics(bg, 1.3)
        alone = lvl.diagnostics(bg, 1.3, strings_only=True)
        assert (alone.n_p_plain, alone.n_p_weighted, alone.n_near_tie) == \
            (full.n_p_plain, full.n_p_weighted, full.n_near_tie), name
        assert torch.equal(torch.sort(alone.pierced)[0], torch.sort(full.pierced)[0]), name
        if name == "pi":
            assert full.n_near_tie > 0


@pytest.mark.parametrize("vacuum", [4, 20])
def test_per_cell_fp32_double_path_cells(axs, orc, vacuum):
    """per_cell_fp32 on a field with exact zeros (|psi|^2 = 0: the double path)
    and a false-vacuum block; at 20^3 the block overflows the energy kernel's
    per-chunk queue, which then searches the chunk again. Counts, the velocity
    count and the pierced set equal the FP64 per-cell pass; sums to 2e-6."""
    n = 48
    v = orc.fourier_ic_state(n, 6.0, seed=12)
    v[2:] = 0.2 * np.random.default_rng(4).standard_normal((2, n, n, n))
    zs = np.random.default_rng(5).integers(0, n, size=(80, 3))
    v[:2, zs[:, 0], zs[:, 1], zs[:, 2]] = 0.0
    v[:, 8:8 + vacuum, 8:8 + vacuum, 8:8 + vacuum] = 0.0
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lvl = axs.PeriodicLevel(n, 0.5, dtype=torch.float32, pierced_capacity=3 * n ** 3)
    lvl.set_state(_dev(v.astype(np.float32)))
    ref = lvl.diagnostics(bg, 1.3)
    fast = lvl.diagnostics(bg, 1.3, per_cell_fp32=True)
    assert (fast.n_p_plain, fast.n_p_weighted, fast.vel_count, fast.n_near_tie) == \
        (ref.n_p_plain, ref.n_p_weighted, ref.vel_count, ref.n_near_tie)
    assert torch.equal(torch.sort(fast.pierced)[0], torch.sort(ref.pierced)[0])
    np.testing.assert_allclose(fast.energy_sums, ref.energy_sums, rtol=2e-6)
    assert fast.energy_sums[13] == ref.energy_sums[13] == n ** 3  # every cell counted once
    assert fast.mean_gamma_sq_v_sq == pytest.approx(ref.mean_gamma_sq_v_sq, rel=1e-5)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_network_scalars_row_matches_oracle(axs, orc, dtype):
    """The 24-column network_scalars.dat row (counts, xi, m_r/H, the 12
    normalised energies, volumes, <gamma^2 v^2>, <gamma>, the velocity corner
    count and the two tensions) of an evolved Fourier-IC level against the
    oracle's restatement of specific_post_timestep's host algebra on the same
    field. FP64: to 1e-12. FP32 fields: the oracle's FP32 build on the GPU's
    own FP32 state; the FLOAT build holds R, lambda, R'/R and m_r as float
    while the GPU's diagnostics take them in double, so the columns agree to
    1e-6 there (counts still exactly)."""
    from axion_strings_adaptive_gb300 import output
    n, dx, dt, steps = 48, 0.5, 0.1, 30
    v = orc.fourier_ic_state(n, orc.strict_cutoff(n / 4), seed=77)
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lv = axs.PeriodicLevel(n, dx, dtype=dtype)
    lv.set_state(torch.from_numpy(v).cuda())
    lv.advance(bg, 1.0, 0.0, dt, steps)
    lv.device_status()
    tau = 1.0 + steps * dt
    d = lv.diagnostics(bg, tau)
    assert d.n_p_plain > 0
    row = np.array(output.network_scalars_row(d, 1.0 / bg.H_over_mr_direct(tau)), dtype=np.float64)
    got_state = lv.get_state().cpu().numpy()
    ref = orc.network_scalars_row(got_state, dx, orc.background(a_inv=2.0, c0=1.0, lambda_scale=2.0), tau)
    assert row.shape == ref.shape == (24,)
    # integer columns (counts) exactly; the rest to 1e-12 relative
    for q in (0, 1, 21):
        assert row[q] == ref[q], output.NETWORK_COLUMNS[q]
    np.testing.assert_allclose(row, ref, rtol=1e-12 if dtype == torch.float64 else 1e-6, atol=0)
