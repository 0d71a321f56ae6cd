"""The C++ host side (host/axs_level.hpp, driven by host/level_demo.cpp) over
the same C ABI: a fused-RK4 run and its post-timestep diagnostics equal the
Python host path bit for bit."""
import json
import os
import subprocess

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_cpp_host_matches_python_host(axs, tmp_path, prec):
    from axion_strings_adaptive_gb300 import _build, ic
    n, steps = 32, 20
    dtype = torch.float64 if prec == "f64" else torch.float32
    s0 = ic.fourier_state(n, ic.strict_cutoff(n / 4), seed=31)
    s0[2:] = 0.05 * torch.randn_like(s0[2:])
    icf, out = tmp_path / "ic.bin", tmp_path / "out.bin"
    s0.cpu().numpy().astype(np.float64).tofile(icf)
    cmd = [_build.DEMO_PATH, prec, str(n), str(n), str(n), "0.5", "2.0", "1.0", "2.0", "1.0", "0.1", str(steps),
           str(icf), str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    got = np.fromfile(out, dtype=np.float64 if prec == "f64" else np.float32).reshape(4, n, n, n)

    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    lvl = axs.AxionStringsLevel(n, 0.5, bg, tau_i=1.0, dtype=dtype)
    lvl.level.set_state(s0.to(dtype))
    lvl.advance(0.1, steps)
    ref = lvl.specific_post_timestep(want_list=False)
    np.testing.assert_array_equal(got, lvl.level.get_state().cpu().numpy())
    assert (d["n_p_plain"], d["n_p_weighted"], d["vel_count"]) == (ref.n_p_plain, ref.n_p_weighted, ref.vel_count)
    assert d["energy_sums"] == list(ref.energy_sums)
    assert d["xi_plain"] == ref.xi_plain and d["tau"] == pytest.approx(3.0)
