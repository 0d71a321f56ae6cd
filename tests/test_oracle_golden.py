"""Pin the CPU oracle (C restatement) against golden vectors produced by the
reference's own code (tests/golden/make_golden.py) -- CPU only.

Mirrors the reference's unit tests: test_plaquette_winding.cpp,
test_energy.cpp, test_velocity.cpp, test_masking.cpp, test_background.cpp,
test_xi_formula.cpp, test_flat_background.cpp,
test_pre_evolution_background.cpp, plus field-level RHS / string finder /
energy / velocity / Fourier-IC fixtures.
"""
import ctypes as C

import numpy as np
import pytest


def test_plaquette_winding_kats(orc, golden):
    g = golden("kats.npz")
    w = orc.plaquette_winding_batch(g["winding_theta"])
    np.testing.assert_array_equal(w, g["winding_w"])
    # the reference's own explicit answers (test_plaquette_winding.cpp:12-53)
    assert list(g["winding_w"][:8]) == [1, -1, 0, 0, 1, 0, 2, 1]


def test_wrap_angle_diff(orc, golden):
    g = golden("kats.npz")
    out = np.array([orc.lib().oracle_wrap_angle_diff(x) for x in g["wrap_in"]])
    np.testing.assert_array_equal(out, g["wrap_out"])


def test_energy_pointwise(orc, golden):
    g = golden("kats.npz")
    inp = np.ascontiguousarray(g["energy_in"])
    out = np.zeros((inp.shape[0], 6))
    orc.lib().oracle_energy_pointwise(orc._p(inp), inp.shape[0], orc._p(out))
    np.testing.assert_array_equal(out, g["energy_out"])
    # vacuum psi = R, Pi = R' has zero energy density (test_energy.cpp:15-34)
    assert np.all(np.abs(out[:4, 0]) <= 1e-10)


def test_masking(orc, golden):
    g = golden("kats.npz")
    L = orc.lib()
    for a, wref, dref in zip(g["mask_in"], g["mask_weight"], g["mask_adot"]):
        assert L.oracle_masking_weight(int(a[0]), a[1], a[2], a[3], a[6]) == wref
        d = L.oracle_masked_a_dot(int(a[0]), *a[1:])
        assert d == dref or (np.isnan(d) and np.isnan(dref))


def test_velocity(orc, golden):
    g = golden("kats.npz")
    L = orc.lib()
    for p, ref in zip(g["vel_psi_in"], g["vel_psi_out"]):
        assert L.oracle_gamma_sq_v_sq_from_psi_literal(*p) == ref
    for p, ref in zip(g["vel_phi_in"], g["vel_phi_out"]):
        assert L.oracle_gamma_sq_v_sq_from_phi(*p) == ref
    # literal psi form equals the phi form (test_velocity.cpp:22-52)
    for p, lit in zip(g["vel_psi_in"], g["vel_psi_out"]):
        psi1, psi2, Pi1, Pi2, R, tau, b_inv, m_r = p
        ibt = 1.0 / (b_inv * tau)
        phi = L.oracle_gamma_sq_v_sq_from_phi(psi1 / R, psi2 / R, (Pi1 - ibt * psi1) / R ** 2,
                                              (Pi2 - ibt * psi2) / R ** 2, m_r)
        assert phi == pytest.approx(lit, rel=1e-9)


def test_background(orc, golden):
    g = golden("kats.npz")
    for cfg, rows in zip(g["bg_cfg"], g["bg_out"]):
        bg = orc.background(a_inv=cfg[0], c0=cfg[1], c1=cfg[2], tau_switch=cfg[3], has_switch=bool(cfg[4]))
        vals = orc.background_eval(bg, g["bg_tau"])
        np.testing.assert_allclose(vals[:, 0], rows[:, 0], rtol=1e-15)  # R
        np.testing.assert_allclose(vals[:, 1], rows[:, 1], rtol=1e-15)  # R'
        np.testing.assert_allclose(vals[:, 2], rows[:, 2], rtol=1e-15)  # curvature
        np.testing.assert_allclose(vals[:, 3], rows[:, 3], rtol=1e-15)  # lambda
        np.testing.assert_allclose(vals[:, 4], rows[:, 4], rtol=1e-15)  # H
        # H/m_r closed form == direct for no-switch runs (test_background.cpp:15-51)
        if not cfg[4]:
            np.testing.assert_allclose(rows[:, 5], rows[:, 6], rtol=1e-12)
    for (a_inv, c0, l), tau in zip(g["bg_log_in"], g["bg_log_tau"]):
        bg = orc.background(a_inv=a_inv, c0=c0)
        assert orc.lib().oracle_bg_tau_from_log_mr_over_h(C.byref(bg), l) == pytest.approx(tau, rel=1e-15)


def test_flat_and_pre_evolution_background(orc, golden):
    g = golden("kats.npz")
    for a, m in enumerate((1.0, 2.3, 0.7)):
        for b, t in enumerate((0.0, 0.5, 1.0, 10.0, 100.0)):
            v = orc.background_eval(orc.background(kind=orc.BG_FLAT, m_r=m), t)[0]
            np.testing.assert_array_equal([v[0], v[1], v[2], v[3]], g["flat_out"][a, b])
    for a, gp in enumerate((0.5, 1.0, 3.0)):
        for b, t in enumerate((-2.0, -0.3, 0.0, 0.7, 4.0)):
            v = orc.background_eval(orc.background(kind=orc.BG_PRE, gamma_pre=gp), t)[0]
            np.testing.assert_allclose([v[0], v[1], v[2], v[3]], g["pre_out"][a, b, :4], rtol=1e-15)
            assert g["pre_out"][a, b, 4] == pytest.approx(gp, rel=1e-9)  # m_r/H = gamma_pre


def test_xi_formula(orc, golden):
    g = golden("kats.npz")
    L = orc.lib()
    for x, xi, xil, inv in zip(g["xi_in"], g["xi_out"], g["xi_len_out"], g["xi_inv_out"]):
        assert L.oracle_xi_from_plaquette_count(*x) == xi
        assert L.oracle_xi_from_comoving_length((2 / 3) * x[0] * x[1], *x[2:]) == xil
        assert L.oracle_plaquette_count_for_target_xi(0.7, 64, x[2], x[3], x[4]) == inv


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["rand", "ic"])
def test_fields(orc, golden, prec, box):
    g = golden(f"fields_{prec}.npz")
    dx, kappa, lam, R2, R, RpR, m_r = g["params"]
    st = g[f"{box}_state"]
    ng = 2
    fab = orc.to_fab(np.ascontiguousarray(st), ng)
    # RHS: bit-exact (same expressions, no contraction)
    np.testing.assert_array_equal(orc.from_fab(orc.rhs(fab, ng, dx, kappa, lam, R2), ng), g[f"{box}_rhs"])
    # string finder: windings and counts bit-exact
    pl, wt, w = orc.count_plaquettes(fab, ng, want_windings=True)
    np.testing.assert_array_equal(w, g[f"{box}_windings"])
    assert (pl, wt) == tuple(g[f"{box}_counts"])
    assert orc.count_plaquettes(fab, ng, mask=g[f"{box}_mask"]) == tuple(g[f"{box}_counts_masked"])
    # energy sums (reference: plain sequential sums; oracle: compensated)
    for scheme in range(3):
        e = orc.energy_sums(fab, ng, dx, R, lam, RpR, scheme, 0.8)
        np.testing.assert_allclose(e, g[f"{box}_energy_sums"][scheme], rtol=1e-12, atol=0)
        tot = orc.normalise_energy(e, float(np.prod(st.shape[1:])))
        np.testing.assert_allclose(tot, g[f"{box}_energy_total"][scheme], rtol=1e-12)
    em = orc.energy_sums(fab, ng, dx, R, lam, RpR, 1, 0.8, mask=g[f"{box}_mask"])
    np.testing.assert_allclose(em, g[f"{box}_energy_sums_masked"], rtol=1e-12)
    vs, vc = orc.velocity(fab, ng, R, RpR, m_r)
    assert vc == int(g[f"{box}_velocity"][1])
    assert vs == pytest.approx(g[f"{box}_velocity"][0], rel=1e-12)


def test_fourier_ic(orc, golden):
    g = golden("fourier_ic.npz")
    for tag in ("a", "b"):
        nx, ny, nz, kmax, seed, comp = g[f"{tag}_args"]
        f = orc.fourier_ic_component(int(nx), int(ny), int(nz), kmax, 0.5, int(seed), int(comp))
        np.testing.assert_allclose(f, g[f"{tag}_field"], rtol=0, atol=1e-13)
    L = orc.lib()
    for x, h in zip(g["hash_in"], g["hash_out"]):
        assert L.oracle_hash_u64(int(x)) == int(h)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["rand", "ic"])
def test_tagger_matches_reference(orc, golden, prec, box):
    """StringTagger::operator() (StringTagger.hpp:117-151): plaquette, Laplacian and
    radial-gradient criteria, restated in the oracle, against the reference's own
    tagger on the same boxes."""
    g = golden("tagging.npz")
    fab = orc.to_fab(np.ascontiguousarray(g[f"{prec}_{box}_state"]), 2)
    for t, (gt, rt) in enumerate(g["thresholds"]):
        tags = orc.tag_cells(fab, 2, 0.5, gt, rt, 0)
        np.testing.assert_array_equal(tags, g[f"{prec}_{box}_tags"][t].astype(np.uint8))


def test_tag_buffer_is_a_periodic_cube(orc):
    """n_error_buf: every cell within nbuf cells (a cube, periodic wrap) of a tag."""
    rng = np.random.default_rng(4)
    v = rng.standard_normal((4, 9, 10, 12))
    fab = orc.to_fab(v, 2)
    base = orc.tag_cells(fab, 2, 0.5, 1e300, 1e300, 0)
    for nb in (1, 2):
        got = orc.tag_cells(fab, 2, 0.5, 1e300, 1e300, nb)
        ref = np.zeros_like(base)
        for dz in range(-nb, nb + 1):
            for dy in range(-nb, nb + 1):
                for dx in range(-nb, nb + 1):
                    ref |= np.roll(base, (dz, dy, dx), axis=(0, 1, 2))
        np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["cube", "odd"])
@pytest.mark.parametrize("scheme", [0, 2])
def test_spectrum_matches_reference(orc, golden, prec, box, scheme):
    """fill_masked_a_dot_buffer + compute_spectrum (MaskedFieldBuffer.hpp,
    SpectrumKernel.hpp:53-153) restated in the oracle against the reference's own
    code: buffer bit-exact, shell averages / counts / totals to FFT rounding."""
    g = golden("spectrum.npz")
    key = f"{prec}_{box}_s{scheme}"
    fab = orc.to_fab(np.ascontiguousarray(g[f"{prec}_{box}_state"]), 2)
    buf = orc.masked_a_dot_buffer(fab, 2, scheme, 0.8, 1.1)
    np.testing.assert_array_equal(buf, g[f"{key}_buffer"])
    sp = orc.spectrum(buf)
    cnt = g[f"{key}_shell_count"]
    np.testing.assert_array_equal(sp["shell_count"], cnt)
    avg = np.where(cnt > 0, sp["shell_sum"] / np.maximum(cnt, 1), 0.0)
    tol = 1e-12 if prec == "f64" else 1e-6
    np.testing.assert_allclose(avg, g[f"{key}_shell_average"], rtol=tol, atol=tol * np.abs(avg).max())
    tot = g[f"{key}_totals"]
    assert sp["full_cube_energy"] == pytest.approx(tot[0], rel=tol)
    assert sp["inscribed_sphere_energy"] == pytest.approx(tot[1], rel=tol)
    # MultiFab::Dot returns amrex::Real: the FLOAT build rounds the sum to float
    assert float((buf.astype(np.float64) ** 2).sum()) == pytest.approx(tot[2], rel=1e-12 if prec == "f64" else 1e-7)
