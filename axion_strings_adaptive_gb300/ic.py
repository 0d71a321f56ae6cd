"""Seeded Fourier-mode initial data (FourierIC.hpp:82-130) on the device.

The half spectrum is filled by the library (``axs_fourier_spectrum``: SplitMix64
hash of (seed, component, i, j, k), Box-Muller, modes 0 < k^2 <= k_max^2 in
integer mode-index units); the inverse real FFT (torch.fft, FFTW c2r
convention) and the real-space rescale to the target mean square follow
FourierIC.hpp:118-129. Pi = 0 (AxionStringsLevel.cpp:817).
"""
from __future__ import annotations

import math

import torch

from . import _lib as L


def strict_cutoff(n_max: float) -> float:
    """k_max_cells that realises the strict |n| < n_max under the reference's
    inclusive rule k^2 <= k_max_cells^2 (k^2 is an integer)."""
    return math.sqrt(n_max * n_max - 0.5)


def fourier_component(n, k_max_cells: float, seed: int, comp_seed_offset: int, target_mean_square: float = 0.5,
                      device="cuda", stream=None) -> torch.Tensor:
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    spec = torch.empty((nz, ny, nx // 2 + 1, 2), dtype=torch.float64, device=device)
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream.cuda_stream
    L.call("axs_fourier_spectrum", spec.data_ptr(), nx, ny, nz, float(k_max_cells), int(seed) & (2 ** 64 - 1),
           int(comp_seed_offset), s)
    field = torch.fft.irfftn(torch.view_as_complex(spec), s=(nz, ny, nx))
    del spec
    ms = float(torch.dot(field.reshape(-1), field.reshape(-1))) / field.numel()
    if ms > 0.0:
        field.mul_(math.sqrt(target_mean_square / ms))
    return field


def fourier_state(n, k_max_cells: float, seed: int, target_mean_square: float = 0.5, dtype=torch.float64,
                  device="cuda") -> torch.Tensor:
    """(4, nz, ny, nx) state: psi1/psi2 from component seeds 0/1
    (AxionStringsLevel.cpp:810-815), Pi1 = Pi2 = 0."""
    nx, ny, nz = (n, n, n) if isinstance(n, int) else n
    out = torch.zeros((4, nz, ny, nx), dtype=dtype, device=device)
    out[0] = fourier_component(n, k_max_cells, seed, 0, target_mean_square, device).to(dtype)
    out[1] = fourier_component(n, k_max_cells, seed, 1, target_mean_square, device).to(dtype)
    return out
