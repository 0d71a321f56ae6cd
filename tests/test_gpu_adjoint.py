"""Hand-written adjoint of the fused RK4 step behind torch.autograd, through
the C ABI: directional derivatives against central finite differences, the
lambda0 gradient, checkpoint-interval invariance, and FP32 against the FP64
adjoint (the differentiation configuration at reduced size)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ic(n, seed, dtype):
    from axion_strings_adaptive_gb300 import ic
    s = ic.fourier_state(n, ic.strict_cutoff(max(2.0, n / 4)), seed=seed, dtype=torch.float64)
    g = torch.Generator(device="cuda").manual_seed(seed)
    s[2:] = 0.05 * torch.randn((2,) + tuple(s.shape[1:]), generator=g, device="cuda", dtype=torch.float64)
    return s.to(dtype)


def _loss(axs, s, lam, spec):
    from axion_strings_adaptive_gb300.adjoint import string_core_loss
    return string_core_loss(s, lam, spec)


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 12, 10)])
def test_adjoint_matches_central_differences_fp64(axs, shape):
    from axion_strings_adaptive_gb300.adjoint import EvolutionSpec
    nx, ny, nz = shape
    spec = EvolutionSpec(dx=0.5, dt=0.1, nsteps=6, c0=1.0, checkpoint_every=4)
    from axion_strings_adaptive_gb300 import ic
    s0 = torch.zeros((4, nz, ny, nx), dtype=torch.float64, device="cuda")
    s0[0] = ic.fourier_component((nx, ny, nz), 3.0, 11, 0).cuda()
    s0[1] = ic.fourier_component((nx, ny, nz), 3.0, 11, 1).cuda()
    gen = torch.Generator(device="cuda").manual_seed(17)
    s0[2:] = 0.05 * torch.randn(s0[2:].shape, generator=gen, device="cuda", dtype=torch.float64)
    lam = torch.tensor(2.0, dtype=torch.float64)
    x = s0.clone().requires_grad_(True)
    lv = lam.clone().requires_grad_(True)
    L0 = _loss(axs, x, lv, spec)
    L0.backward()
    g = x.grad.clone()
    # central differences along unit-norm random directions (the loss has sharp
    # features near string cores, so the step stays far inside its linear range)
    rng = torch.Generator(device="cuda").manual_seed(3)
    eps = 1e-5
    for _ in range(4):
        d = torch.randn(s0.shape, generator=rng, device="cuda", dtype=torch.float64)
        d /= d.norm()
        fd = (float(_loss(axs, s0 + eps * d, lam, spec)) - float(_loss(axs, s0 - eps * d, lam, spec))) / (2 * eps)
        ad = float((g * d).sum())
        assert ad == pytest.approx(fd, rel=1e-6, abs=1e-7 * float(g.norm())), (ad, fd)
    fd_l = (float(_loss(axs, s0, lam + 1e-6, spec)) - float(_loss(axs, s0, lam - 1e-6, spec))) / 2e-6
    assert float(lv.grad) == pytest.approx(fd_l, rel=2e-6, abs=1e-9)


def test_checkpoint_interval_does_not_change_gradients(axs):
    from axion_strings_adaptive_gb300.adjoint import EvolutionSpec
    s0 = _ic(16, 5, torch.float64)
    grads = []
    for k in (1, 3, 7):
        spec = EvolutionSpec(nsteps=7, checkpoint_every=k)
        x = s0.clone().requires_grad_(True)
        lv = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
        _loss(axs, x, lv, spec).backward()
        grads.append((x.grad.clone(), float(lv.grad)))
    for g, l in grads[1:]:
        assert torch.equal(g, grads[0][0]) and l == grads[0][1]


def test_differentiation_config_reduced(axs):
    """Differentiation configuration (FP32, c0 = 1, lambda0 = 2, checkpoints, loss =
    string-core proxy + axion kinetic energy) at 48^3 and 40 steps: FP32 adjoint
    against central differences (eps = 1e-3) on random directions and against
    the FP64 adjoint."""
    from axion_strings_adaptive_gb300.adjoint import EvolutionSpec
    spec = EvolutionSpec(dx=0.5, dt=0.1, nsteps=40, c0=1.0, checkpoint_every=10)
    s64 = _ic(48, 21, torch.float64)
    out = {}
    for dt_ in (torch.float32, torch.float64):
        x = s64.to(dt_).clone().requires_grad_(True)
        lv = torch.tensor(2.0, dtype=dt_, requires_grad=True)
        _loss(axs, x, lv, spec).backward()
        out[dt_] = (x.grad.double(), float(lv.grad))
    g32, l32 = out[torch.float32]
    g64, l64 = out[torch.float64]
    rel = float((g32 - g64).norm() / g64.norm())
    assert rel < 1e-3, rel
    assert l32 == pytest.approx(l64, rel=1e-3)
    # central differences (eps = 1e-3) along unit-norm random directions, the
    # loss evaluated by the FP64 evolution
    rng = torch.Generator(device="cuda").manual_seed(9)
    lam = torch.tensor(2.0, dtype=torch.float64)
    eps = 1e-3
    for _ in range(3):
        d = torch.randn(s64.shape, generator=rng, device="cuda", dtype=torch.float64)
        d /= d.norm()
        fd = (float(_loss(axs, s64 + eps * d, lam, spec)) - float(_loss(axs, s64 - eps * d, lam, spec))) / (2 * eps)
        ad = float((g32 * d).sum())
        assert ad == pytest.approx(fd, rel=1e-2, abs=1e-3 * float(g64.norm())), (ad, fd)
