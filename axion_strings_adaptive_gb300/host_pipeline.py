"""Host-buffer stepping with copies overlapped with compute.

A caller that keeps its fields in host memory (a CPU code handing boxes to the
GPU, or a stream of independent realisations) pays a host->device copy of each
input and a device->host copy of each result per call. :class:`HostStepPipeline`
runs those copies on their own streams into rotating device staging buffers,
so that the input of call s+1 and the result of call s-1 move while call s
computes (H2D and D2H also overlap each other: the link is full duplex).
Every call is: pinned host state -> H2D -> ``axs_level_import_fab`` ->
``axs_level_rk4_advance`` -> ``axs_level_export_fab`` -> D2H.
"""
from __future__ import annotations

import torch

from .background import Background
from .level import PeriodicLevel


class HostStepPipeline:
    def __init__(self, level: PeriodicLevel, depth: int = 2):
        dev = level.state.device
        self.level = level
        self.depth = max(1, int(depth))
        shape = (4, level.nz, level.ny, level.nx)
        self.staging = [torch.empty(shape, dtype=level.dtype, device=dev) for _ in range(self.depth)]
        self.h2d, self.comp, self.d2h = (torch.cuda.Stream(device=dev) for _ in range(3))
        self._h2d_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._comp_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._d2h_done = [torch.cuda.Event() for _ in range(self.depth)]
        self._used = [False] * self.depth
        self._k = 0

    def submit(self, host_in: torch.Tensor, host_out: torch.Tensor, bg: Background, tau_i: float, t0: float,
               dt: float, nsteps: int = 1) -> None:
        """Queue one call: host_in (pinned, (4, nz, ny, nx)) advanced nsteps -> host_out (pinned)."""
        slot = self._k % self.depth
        self._k += 1
        buf = self.staging[slot]
        if self._used[slot]:
            self.h2d.wait_event(self._d2h_done[slot])  # the slot's previous result has left
        self._used[slot] = True
        with torch.cuda.stream(self.h2d):
            buf.copy_(host_in, non_blocking=True)
            self._h2d_done[slot].record(self.h2d)
        self.comp.wait_event(self._h2d_done[slot])
        with torch.cuda.stream(self.comp):
            self.level.import_fab(buf, 0, self.comp)
            self.level.advance(bg, tau_i, t0, dt, nsteps, self.comp)
            self.level.export_fab(buf, 0, self.comp)
            self._comp_done[slot].record(self.comp)
        self.d2h.wait_event(self._comp_done[slot])
        with torch.cuda.stream(self.d2h):
            host_out.copy_(buf, non_blocking=True)
            self._d2h_done[slot].record(self.d2h)

    def join(self, stream: torch.cuda.Stream | None = None) -> None:
        """Make `stream` (default: the current stream) wait for everything queued."""
        s = stream or torch.cuda.current_stream()
        for st in (self.h2d, self.comp, self.d2h):
            s.wait_stream(st)
