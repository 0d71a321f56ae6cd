"""Host-buffer stepping with copies overlapped with compute.

A caller that keeps its fields in host memory (a CPU code handing boxes to the
GPU, or a stream of independent realisations) pays a host->device copy of each
input and a device->host copy of each result per call. :class:`HostStepPipeline`
rotates over `depth` device levels: the upload of call s+1, the compute of call
s and the download of call s-1 use different levels, so the two copy
directions (the link is full duplex) and the compute overlap. Uploads and
downloads run on streams of their own per level, so a level's scatter or
gather kernel never holds up the copy engine for the next level. Every call is:
pinned host state -> ``axs_level_upload`` (one contiguous DMA copy into the
level's work buffer, then a scatter into the level layout with its periodic
padding) -> ``axs_level_rk4_advance`` -> ``axs_level_download`` (gather into
the work buffer, one contiguous DMA copy) -> pinned host result.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .background import Background
from .level import PeriodicLevel


class HostStepPipeline:
    def __init__(self, level: PeriodicLevel, depth: int = 3):
        self.levels = [level]
        for _ in range(max(1, int(depth)) - 1):
            lv = PeriodicLevel((level.nx, level.ny, level.nz), level.dx, dtype=level.dtype, device=level.state.device,
                               pierced_capacity=1, tile_config=level.tile_config)
            self.levels.append(lv)
        dev = level.state.device
        self.depth = len(self.levels)
        self.comp = torch.cuda.Stream(device=dev)
        self.ups = [torch.cuda.Stream(device=dev) for _ in range(self.depth)]
        self.downs = [torch.cuda.Stream(device=dev) for _ in range(self.depth)]
        self._up_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._comp_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._down_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._used = [False] * self.depth
        self._k = 0

    def submit(self, host_in: torch.Tensor, host_out: torch.Tensor, bg: Background, tau_i: float, t0: float,
               dt: float, nsteps: int = 1) -> None:
        """Queue one call: host_in (pinned, (4, nz, ny, nx)) advanced nsteps -> host_out (pinned)."""
        slot = self._k % self.depth
        self._k += 1
        lv = self.levels[slot]
        up, down = self.ups[slot], self.downs[slot]
        if self._used[slot]:
            up.wait_event(self._down_done[slot])  # the slot's previous result has left
        self._used[slot] = True
        L.call("axs_level_upload", C.byref(lv.c), C.c_void_p(host_in.data_ptr()), up.cuda_stream)
        self._up_done[slot].record(up)
        self.comp.wait_event(self._up_done[slot])
        lv.advance(bg, tau_i, t0, dt, nsteps, self.comp)
        self._comp_done[slot].record(self.comp)
        down.wait_event(self._comp_done[slot])
        L.call("axs_level_download", C.byref(lv.c), C.c_void_p(host_out.data_ptr()), down.cuda_stream)
        self._down_done[slot].record(down)

    def join(self, stream: torch.cuda.Stream | None = None) -> None:
        """Make `stream` (default: the current stream) wait for everything queued."""
        s = stream or torch.cuda.current_stream()
        for st in [self.comp] + self.ups + self.downs:
            s.wait_stream(st)

    def device_status(self) -> None:
        for lv in self.levels:
            lv.device_status()
