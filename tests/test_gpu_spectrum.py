"""Axion power spectrum through the C ABI: masked a_dot buffer + cuFFT R2C +
device shell binning against the reference's own compute_spectrum (golden
fixtures from the reference-built checker), both precisions, schemes None and
B; Parseval on a larger evolved box."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["cube", "odd"])
@pytest.mark.parametrize("scheme", [0, 2])
def test_spectrum_matches_reference(axs, golden, prec, box, scheme):
    from axion_strings_adaptive_gb300.spectrum import spectrum_at
    g = golden("spectrum.npz")
    key = f"{prec}_{box}_s{scheme}"
    v = g[f"{prec}_{box}_state"]
    _, nz, ny, nx = v.shape
    dtype = torch.float64 if prec == "f64" else torch.float32
    lv = axs.PeriodicLevel((nx, ny, nz), 0.5, dtype=dtype)
    lv.set_state(torch.from_numpy(np.ascontiguousarray(v)).cuda())
    sp = spectrum_at(lv, 1.1, 0.0, scheme, 0.8)
    cnt = g[f"{key}_shell_count"]
    ref_avg = g[f"{key}_shell_average"]
    nonempty = np.nonzero(cnt > 0)[0]
    np.testing.assert_array_equal(sp.p, nonempty)
    np.testing.assert_array_equal(sp.shell_count, cnt[nonempty])
    tol = 1e-12 if prec == "f64" else 2e-5
    np.testing.assert_allclose(sp.shell_average, ref_avg[nonempty], rtol=tol, atol=tol * np.abs(ref_avg).max())
    tot = g[f"{key}_totals"]
    assert sp.full_cube_energy == pytest.approx(tot[0], rel=tol)
    assert sp.inscribed_sphere_energy == pytest.approx(tot[1], rel=tol)
    assert sp.real_space_mean_sq * nx * ny * nz == pytest.approx(tot[2], rel=1e-12 if prec == "f64" else 1e-7)


def test_parseval_and_determinism(axs):
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.spectrum import level_spectrum
    n = 128
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lv = axs.PeriodicLevel(n, 0.5, dtype=torch.float32)
    lv.set_state(ic.fourier_state(n, ic.strict_cutoff(n / 4), seed=12).float())
    lv.advance(bg, 1.0, 0.0, 0.1, 30)
    a = level_spectrum(lv, bg, 4.0, axs._lib.MASK_B, 0.8)
    b = level_spectrum(lv, bg, 4.0, axs._lib.MASK_B, 0.8)
    assert a.parseval_full == pytest.approx(a.real_space_mean_sq, rel=1e-5)
    assert a.inscribed_sphere_energy <= a.full_cube_energy
    np.testing.assert_array_equal(a.shell_average, b.shell_average)  # fixed-order reductions
    assert len(a.p) == n // 2 + 1 and a.shell_count.sum() > 0
