"""Pre-evolution -> main handoff and checkpoint/restart through the C ABI:
the device rescale equals the oracle restatement of
apply_pre_evolution_to_main_rescale bit for bit (both precisions); the level
hook moves the clock and background as the reference does; a run restored
from a checkpoint continues bit-identically to an uninterrupted one."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_handoff_rescale_matches_oracle(axs, orc, dtype):
    from axion_strings_adaptive_gb300 import ic
    n = 16
    s = ic.fourier_state(n, 4.0, seed=2)
    s[2:] = 0.2 * torch.randn_like(s[2:])
    s = s.to(dtype)
    pre = axs.Background.pre_evolution(0.7)
    main = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lvl = axs.AxionStringsLevel(n, 0.5, pre, tau_i=0.0, dtype=dtype)
    lvl.level.set_state(s)
    lvl.time = 1.3  # end of the pre-evolution clock
    lvl.apply_pre_evolution_to_main_rescale(main, 1.0, transition_n_periods=2.0)
    vp, vm = pre.values(1.3), main.values(1.0)
    fab = orc.to_fab(s.cpu().numpy(), 2)
    orc.handoff_rescale(fab, 2, vp.R, vp.R_prime, vm.R, vm.R_prime)
    np.testing.assert_array_equal(lvl.level.get_state().cpu().numpy(), orc.from_fab(fab, 2))
    assert lvl.tau == pytest.approx(1.0) and lvl.bg.blend_tau_start == 1.0 and lvl.bg.blend_dtau > 0.0
    assert lvl.bg.blend_lambda_start == vp.lambda_
    lvl.advance(0.1, 3)  # the blended main schedule runs
    lvl.level.device_status()


def test_checkpoint_restart_is_bit_identical(axs, tmp_path):
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.output import load_checkpoint, save_checkpoint
    n = 32
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 4), seed=4).float()
    a = axs.AxionStringsLevel(n, 0.5, bg, tau_i=1.0, dtype=torch.float32)
    a.level.set_state(s0)
    a.advance(0.1, 5)
    save_checkpoint(str(tmp_path / "chk.npz"), a, step=5)
    a.advance(0.1, 7)
    b = axs.AxionStringsLevel(n, 0.5, axs.Background.flat(1.0), tau_i=0.0, dtype=torch.float32)
    assert load_checkpoint(str(tmp_path / "chk.npz"), b) == 5
    assert b.bg == bg and b.tau == pytest.approx(1.5)
    b.advance(0.1, 7)
    assert torch.equal(a.level.get_state(), b.level.get_state())
