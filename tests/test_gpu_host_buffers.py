"""Host-buffer entry points: axs_level_upload / axs_level_download move a
pinned (4, nz, ny, nx) array into / out of the level layout exactly (padding
refreshed), and the overlapped HostStepPipeline gives the same results as
uploading, advancing and downloading one call at a time."""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_upload_download_round_trip(axs, dtype):
    from axion_strings_adaptive_gb300 import _lib as L
    nx, ny, nz = 40, 24, 12
    host = torch.randn((4, nz, ny, nx), dtype=dtype).pin_memory()
    lv = axs.PeriodicLevel((nx, ny, nz), 0.5, dtype=dtype)
    L.call("axs_level_upload", C.byref(lv.c), C.c_void_p(host.data_ptr()), None)
    torch.cuda.synchronize()
    assert torch.equal(lv.get_state().cpu(), host)
    ref = axs.PeriodicLevel((nx, ny, nz), 0.5, dtype=dtype)
    ref.set_state(host.cuda())
    assert torch.equal(lv.state, ref.state)  # same padding as set_state
    out = torch.empty_like(host).pin_memory()
    L.call("axs_level_download", C.byref(lv.c), C.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    assert torch.equal(out, host)


def test_pipeline_matches_serial_calls(axs):
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.host_pipeline import HostStepPipeline
    n = 32
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    ins = [(ic.fourier_state(n, 4.0, seed=s).float()).cpu().pin_memory() for s in range(5)]
    outs = [torch.empty_like(ins[0]).pin_memory() for _ in range(5)]
    lv = axs.PeriodicLevel(n, 0.5, dtype=torch.float32)
    pipe = HostStepPipeline(lv, depth=3)
    for s in range(5):
        pipe.submit(ins[s], outs[s], bg, 1.0, 0.1 * s, 0.1, 2)
    pipe.join()
    torch.cuda.synchronize()
    pipe.device_status()
    for s in range(5):
        ref = axs.PeriodicLevel(n, 0.5, dtype=torch.float32)
        ref.set_state(ins[s].cuda())
        ref.advance(bg, 1.0, 0.1 * s, 0.1, 2)
        assert torch.equal(outs[s], ref.get_state().cpu())
