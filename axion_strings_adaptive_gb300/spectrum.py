"""The axion power spectrum of specific_post_timestep (AxionStringsLevel.cpp:1583-1640).

masked a_dot buffer (libaxs_gb300: ``axs_level_masked_a_dot``) -> unnormalised
forward R2C (cuFFT through torch.fft) -> shell binning (``axs_spectrum_bin``),
then the host algebra of the reference: shell averages of non-empty shells,
Parseval cross-checks and the k/H axis of axion_spectrum.dat.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math

import numpy as np
import torch

from . import _lib as L
from .background import Background
from .level import _DT, PeriodicLevel, _stream_ptr


@dataclasses.dataclass
class Spectrum:
    p: np.ndarray               # shell index of every non-empty shell
    shell_average: np.ndarray   # 4 pi <p^2 |X_p|^2> per shell (getSpectrum's raw output)
    shell_count: np.ndarray
    full_cube_energy: float     # sum over all modes of |X_p|^2
    inscribed_sphere_energy: float
    real_space_mean_sq: float   # <buffer^2>
    parseval_full: float        # full_cube_energy / N^2 (equals real_space_mean_sq)
    parseval_inscribed: float
    k_over_H: np.ndarray        # 2 pi q / (L H), q = row index among the non-empty shells


def level_spectrum(level: PeriodicLevel, bg: Background, tau: float, masking_scheme: int = L.MASK_NONE,
                   threshold: float = 0.8, stream=None) -> Spectrum:
    """The spectrum of the level's masked a_dot at conformal time tau."""
    v = bg.values(tau)
    return spectrum_at(level, v.R, v.H, masking_scheme, threshold, stream)


def spectrum_at(level: PeriodicLevel, R: float, H: float = 0.0, masking_scheme: int = L.MASK_NONE,
                threshold: float = 0.8, stream=None) -> Spectrum:
    """The same with R(tau) and H(tau) given directly."""
    nx, ny, nz = level.nx, level.ny, level.nz
    dev = level.state.device
    b = C.c_int64()
    L.call("axs_spectrum_scratch_bytes", nx, ny, nz, C.byref(b))
    scratch = torch.empty(max(b.value, 8 * 4096), dtype=torch.uint8, device=dev)
    buf = torch.empty((nz, ny, nx), dtype=level.dtype, device=dev)
    sums = torch.zeros(3, dtype=torch.float64, device=dev)  # sum_sq, full, inscribed
    L.call("axs_level_masked_a_dot", C.byref(level.c), int(masking_scheme), float(threshold), float(R),
           buf.data_ptr(), sums.data_ptr(), scratch.data_ptr(), scratch.numel(), _stream_ptr(stream))
    X = torch.fft.rfftn(buf).contiguous()  # cuFFT may hand back permuted strides
    S = max(nx, ny, nz) // 2 + 1
    shell_sum = torch.zeros(S, dtype=torch.float64, device=dev)
    shell_cnt = torch.zeros(S, dtype=torch.int64, device=dev)
    L.call("axs_spectrum_bin", X.data_ptr(), _DT[level.dtype], nx, ny, nz, shell_sum.data_ptr(), shell_cnt.data_ptr(),
           sums[1:].data_ptr(), scratch.data_ptr(), scratch.numel(), _stream_ptr(stream))
    s_sum, s_cnt, tot = shell_sum.cpu().numpy(), shell_cnt.cpu().numpy(), sums.cpu().numpy()
    nonempty = np.nonzero(s_cnt > 0)[0]
    n_cells = float(nx * ny * nz)
    # axion_spectrum.dat's k_over_H column: 2 pi / (L H) times the row's index
    # among the non-empty shells (AxionStringsLevel.cpp:1735-1760)
    k_per_mode = 2.0 * math.pi / (nx * level.dx * H) if H > 0.0 else 0.0
    return Spectrum(p=nonempty.astype(np.float64), shell_average=s_sum[nonempty] / s_cnt[nonempty],
                    shell_count=s_cnt[nonempty], full_cube_energy=float(tot[1]),
                    inscribed_sphere_energy=float(tot[2]), real_space_mean_sq=float(tot[0]) / n_cells,
                    parseval_full=float(tot[1]) / n_cells ** 2, parseval_inscribed=float(tot[2]) / n_cells ** 2,
                    k_over_H=k_per_mode * np.arange(len(nonempty), dtype=np.float64))
