"""Acceptance checks of the reference that parity alone does not cover
(docs/conventions.md:659-730, docs/STATUS.md:12), run through the C ABI:

* T1 straight string / antistring along z (AxionStringsLevel.cpp:384-476):
  exactly 2 pierced xy plaquettes per z layer, N_p = 2 N_z, before and after
  evolution (the static profile with Pi = (R'/R) psi stays put);
* the 4th-order Laplacian converges at order 4 on a smooth periodic field;
* FP32 evolution tracks FP64 on the precision configuration's physics at a
  reduced size;
* a 1024^3 level (element offsets past 32 bits) evolves a z-only field exactly
  as an 8 x 8 x 1024 column does.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def straight_string_pair(n, nz, dx, R, m_r, RpR):
    """T1 initial data (AxionStringsLevel.cpp:384-476): vortex/antivortex along z,
    separated by L/4 either side of the centre. Samples sit at cell centres
    (i + 1/2) dx, so the cores are put on cell corners -- the centres of
    plaquettes -- to keep every sample off a (phase-undefined) core."""
    L = n * dx
    c = 0.5 * L
    sep = 0.25 * L
    x1, y1 = c - sep, c
    x2, y2 = c + sep, c
    x = (np.arange(n) + 0.5) * dx
    X, Y = np.meshgrid(x, x, indexing="xy")  # [y, x]
    rho1 = np.hypot(X - x1, Y - y1)
    rho2 = np.hypot(X - x2, Y - y2)
    theta = np.arctan2(Y - y1, X - x1) - np.arctan2(Y - y2, X - x2)
    g1 = (m_r * rho1) / np.sqrt((m_r * rho1) ** 2 + 2.0)
    g2 = (m_r * rho2) / np.sqrt((m_r * rho2) ** 2 + 2.0)
    amp = R * g1 * g2
    s = np.zeros((4, nz, n, n))
    s[0] = amp * np.cos(theta)
    s[1] = amp * np.sin(theta)
    s[2] = RpR * s[0]
    s[3] = RpR * s[1]
    return s


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_straight_string_pair_gives_two_plaquettes_per_layer(axs, dtype):
    n, nz, dx = 48, 12, 0.5
    bg = axs.Background.expanding(2.0, 1.0)
    v = bg.values(1.0)
    st = straight_string_pair(n, nz, dx, v.R, v.m_r, v.R_prime_over_R)
    lvl = axs.PeriodicLevel((n, n, nz), dx, dtype=dtype)
    lvl.set_state(torch.from_numpy(st).cuda())
    d0 = lvl.diagnostics(bg, 1.0)
    assert (d0.n_p_plain, d0.n_p_weighted) == (2 * nz, 2 * nz)
    planes = (d0.pierced.cpu().numpy() & 3)
    assert set(planes.tolist()) == {0}  # only xy plaquettes: strings run along z
    lvl.advance(bg, 1.0, 0.0, 0.1, 20)
    lvl.device_status()
    d1 = lvl.diagnostics(bg, 3.0)
    assert (d1.n_p_plain, d1.n_p_weighted) == (2 * nz, 2 * nz)
    # gamma^2 v^2 evaluated at the 8 corners per layer of a near-static pair stays small
    assert d1.vel_count == 8 * nz and d1.mean_gamma_sq_v_sq < 0.5


def test_laplacian_is_fourth_order(axs):
    """rhs_Pi = lap(psi) for kappa = lambda = 0: error of the 13-point stencil on
    sin(2 pi x / L) cos(4 pi y / L) falls as dx^4."""
    L = 8.0
    errs = []
    for n in (16, 32, 64):
        dx = L / n
        x = (np.arange(n)) * dx
        Z, Y, X = np.meshgrid(x[:4], x, x, indexing="ij")
        kx, ky = 2 * math.pi / L, 4 * math.pi / L
        f = np.sin(kx * X) * np.cos(ky * Y)
        exact = -(kx ** 2 + ky ** 2) * f
        st = np.zeros((4, 4, n, n))
        st[0] = f
        t = axs.new_fab((n, n, 4), 2, dtype=torch.float64)
        axs.valid(t, 2).copy_(torch.from_numpy(st).cuda())
        axs.fill_periodic_ghosts(t, 2)
        r = axs.new_fab((n, n, 4), 0, dtype=torch.float64)
        axs.eval_rhs(t, r, 2, 0, dx, axs._lib.RhsCoeffs(0.0, 0.0, 0.0))
        errs.append(float(np.abs(r[2].cpu().numpy() - exact).max()))
    orders = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert all(3.8 < o < 4.3 for o in orders), (errs, orders)


def test_fp32_tracks_fp64(axs):
    """Precision configuration physics (Moore c0 = 2, lambda0 = 2, RD, dx 0.5,
    dt 0.1, IC |n| < N/8) at 128^3 for 40 steps: FP32 total energy within 1e-5
    of FP64, identical string counts."""
    from axion_strings_adaptive_gb300 import ic
    n = 128
    bg = axs.Background.expanding(2.0, 2.0, lambda0=2.0)
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 8), seed=77)
    out = {}
    for dt_ in (torch.float64, torch.float32):
        lv = axs.PeriodicLevel(n, 0.5, dtype=dt_)
        lv.set_state(s0.to(dt_))
        lv.advance(bg, 1.0, 0.0, 0.1, 40)
        lv.device_status()
        out[dt_] = lv.diagnostics(bg, 5.0, want_list=False)
    a, b = out[torch.float64], out[torch.float32]
    rel = abs(b.energy["rho_tot_unscreened"] - a.energy["rho_tot_unscreened"]) / a.energy["rho_tot_unscreened"]
    assert rel < 1e-5
    assert b.n_p_plain == a.n_p_plain


def test_1024_cubed_level_indexes_beyond_32_bits(axs):
    """A 1024^3 FP32 level holds 4.6 G elements per component-major array, past
    32-bit offsets. A field that varies only in z must evolve as the same
    column on an 8 x 8 x 1024 level does, bit for bit in every (x, y), and its
    diagnostics must be the column's times the number of columns."""
    free, _ = torch.cuda.mem_get_info()
    if free < 120 * 2 ** 30:
        pytest.skip("needs ~80 GB of free device memory")
    n = 1024
    bg = axs.Background.expanding(2.0, 2.0, lambda0=2.0)
    z = torch.arange(n, dtype=torch.float64, device="cuda")
    col = torch.stack([1.0 + 0.1 * torch.sin(2 * math.pi * 3 * z / n), 0.1 * torch.cos(2 * math.pi * 5 * z / n),
                       0.02 * torch.sin(2 * math.pi * 2 * z / n), torch.zeros_like(z)]).float()  # (4, nz)
    small = axs.PeriodicLevel((8, 8, n), 0.5, dtype=torch.float32, pierced_capacity=1)
    small.set_state(col[:, :, None, None].expand(4, n, 8, 8))
    big = axs.PeriodicLevel(n, 0.5, dtype=torch.float32, pierced_capacity=1)
    big.set_state(col[:, :, None, None].expand(4, n, n, n))
    for lv in (small, big):
        lv.advance(bg, 1.0, 0.0, 0.1, 2)
        lv.device_status()
    ref = small.valid_view()[:, :, 0, 0]
    got = big.valid_view()
    for c in range(4):
        assert bool((got[c] == ref[c][:, None, None]).all()), c
    # FP64 per-cell terms: every cell's terms are the column's, only the summation order differs
    ds = small.diagnostics(bg, 1.2, want_list=False)
    db = big.diagnostics(bg, 1.2, want_list=False)
    assert ds.n_p_plain == 0 and db.n_p_plain == 0
    scale = (n * n) / 64.0
    np.testing.assert_allclose(np.array(db.energy_sums), scale * np.array(ds.energy_sums), rtol=1e-10)
    del big
    torch.cuda.empty_cache()
