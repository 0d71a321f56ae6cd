"""Ensembles of independent periodic boxes of uneven sizes (the batching path).

:class:`Ensemble` packs its boxes component-major in one state arena and one
stage-buffer arena (the ``axs_ensemble`` layout of include/axs.h), builds the
device table for one tiling, and advances every box together: with the
one-pass fused step (one persistent launch per RK4 step plus one for the
periodic padding; the default for boxes with ny a multiple of 16 and an even
nx) or with two persistent sweep launches per step (any box shape).
``capture(...)`` records a whole run -- the steps plus
per-box diagnostics -- as one CUDA graph; :meth:`Ensemble.autotune` times the
compiled tilings and z-chunk targets (the work each block takes from a box) on
the caller's boxes and keeps the fastest.

Each box evolves exactly as a :class:`~.level.PeriodicLevel` of its size would,
bit for bit: the per-site arithmetic is the same and tiling changes only which
block computes a site.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .background import Background
from .level import _DT, _stream_ptr, summarise


class Ensemble:
    def __init__(self, dims, dx: float, dtype=torch.float32, device="cuda", tile_config: int = 0, z_chunk: int = 0):
        self.dims = [tuple(int(v) for v in d) for d in dims]
        self.nboxes = len(self.dims)
        self.dx, self.dtype = float(dx), dtype
        self._dims_c = (C.c_int32 * (3 * self.nboxes))(*[v for d in self.dims for v in d])
        sb, wb, tb = C.c_int64(), C.c_int64(), C.c_int64()
        L.call("axs_ensemble_sizes", _DT[dtype], self.nboxes, self._dims_c, C.byref(sb), C.byref(wb), C.byref(tb))
        es = torch.finfo(dtype).bits // 8
        self.plane = sb.value // (4 * es)
        self.state = torch.zeros((4, self.plane), dtype=dtype, device=device)
        self.work = torch.zeros((8, self.plane), dtype=dtype, device=device)
        self.table = torch.zeros(tb.value, dtype=torch.uint8, device=device)
        self.c = L.EnsembleC(_DT[dtype], self.nboxes, self._dims_c, self.dx, self.state.data_ptr(),
                             self.work.data_ptr(), self.table.data_ptr(), sb.value, wb.value, tb.value)
        self.boxes = []
        for b in range(self.nboxes):
            lay = L.EnsembleBox()
            L.call("axs_ensemble_box_layout", _DT[dtype], self.nboxes, self._dims_c, b, C.byref(lay))
            self.boxes.append(lay)
        nbytes = C.c_int64()
        L.call("axs_ensemble_diagnostics_scratch_bytes", self.nboxes, self._dims_c, C.byref(nbytes))
        self._scratch = torch.zeros(nbytes.value, dtype=torch.uint8, device=device)
        self._results = torch.zeros((self.nboxes, C.sizeof(L.DiagResult)), dtype=torch.uint8, device=device)
        self.plan = L.EnsemblePlan()
        self.init(tile_config, z_chunk)

    # ------------------------------------------------------------------ layout
    def init(self, tile_config: int = 0, z_chunk: int = 0, stream=None) -> None:
        """(Re)build the device table for one tiling; host-synchronous."""
        self.plan.tile_config = int(tile_config)
        self.plan.z_chunk = int(z_chunk)
        L.call("axs_ensemble_init", C.byref(self.c), C.byref(self.plan), _stream_ptr(stream))

    def tile_configs(self) -> list:
        lib = L.lib()
        d = _DT[self.dtype]
        return [(i, lib.axs_ensemble_tile_config_name(d, i).decode())
                for i in range(1, lib.axs_ensemble_tile_config_count(d) + 1)]

    def box_view(self, b: int, arena: torch.Tensor | None = None) -> torch.Tensor:
        """(ncomp, nz, ny, nx) view of box b's valid cells in an arena (default: the state)."""
        t = self.state if arena is None else arena
        nx, ny, nz = self.dims[b]
        lay = self.boxes[b]
        blk = t[:, lay.base:lay.base + nz * lay.kstride].view(t.shape[0], nz, ny + 4, lay.jstride)
        return blk[:, :, lay.y_offset:lay.y_offset + ny, lay.x_offset:lay.x_offset + nx]

    def set_box(self, b: int, valid_cells: torch.Tensor) -> None:
        self.box_view(b).copy_(valid_cells.to(device=self.state.device, dtype=self.dtype))

    def get_box(self, b: int) -> torch.Tensor:
        return self.box_view(b).clone()

    def fill_ghosts(self, stream=None) -> None:
        L.call("axs_ensemble_fill_ghosts", C.byref(self.c), _stream_ptr(stream))

    @property
    def n_sites(self) -> int:
        return sum(nx * ny * nz for nx, ny, nz in self.dims)

    # ------------------------------------------------------------------ evolution
    def advance(self, bg: Background, tau_i: float, t0: float, dt: float, nsteps: int, stream=None) -> None:
        """nsteps RK4 steps of every box (the plan's tiling); asynchronous."""
        L.call("axs_ensemble_rk4_advance", C.byref(self.c), C.byref(self.plan), C.byref(bg.to_c()), float(tau_i),
               float(t0), float(dt), int(nsteps), _stream_ptr(stream))

    def device_status(self, stream=None) -> None:
        L.call("axs_ensemble_device_status", C.byref(self.c), _stream_ptr(stream))

    def diagnostics_async(self, bg: Background, tau: float, masking_scheme: int = L.MASK_A,
                          threshold: float = 0.8, per_cell_fp32: bool = False, stream=None) -> None:
        """Per-box diagnostics into the device result array (no host sync)."""
        v = bg.values(tau)
        rpr = 0.0 if bg.kind == L.BG_FLAT else v.R_prime_over_R
        self._params = L.DiagParams(self.dx, v.R, v.lambda_, rpr, v.m_r, masking_scheme, threshold,
                                    L.BOUNDARY_PERIODIC, 1, 1, 1, int(per_cell_fp32))
        L.call("axs_ensemble_diagnostics", C.byref(self.c), C.byref(self._params), self._results.data_ptr(),
               self._scratch.data_ptr(), self._scratch.numel(), _stream_ptr(stream))

    def results(self, bg: Background, tau: float) -> list:
        """Host summaries of the last per-box diagnostics (synchronises)."""
        host = self._results.cpu().numpy()
        v = bg.values(tau)
        out = []
        for b, (nx, ny, nz) in enumerate(self.dims):
            r = L.DiagResult.from_buffer_copy(host[b].tobytes())
            out.append(summarise(r, n_cells=nx * ny * nz, dx=self.dx, L_tilde=nx * self.dx, a_inv=bg.a_inv, tau=tau,
                                 R=v.R, pierced=None))
        return out

    def diagnostics(self, bg: Background, tau: float, **kw) -> list:
        self.diagnostics_async(bg, tau, **kw)
        return self.results(bg, tau)

    def capture(self, bg: Background, tau_i: float, t0: float, dt: float, nsteps: int,
                diagnostics: bool = True, per_cell_fp32: bool = False) -> torch.cuda.CUDAGraph:
        """Record nsteps RK4 steps of every box (plus per-box diagnostics at the
        end, per-cell terms in FP64 or, with per_cell_fp32, in FP32) as one CUDA
        graph; replay it with ``graph.replay()``."""
        # warm-up outside the capture (module loading, kernel attributes), state restored
        saved = self.state.clone()
        side = torch.cuda.Stream(device=self.state.device)
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.advance(bg, tau_i, t0, dt, 1, side)
            if diagnostics:
                self.diagnostics_async(bg, tau_i + t0 + nsteps * dt, per_cell_fp32=per_cell_fp32, stream=side)
        torch.cuda.current_stream().wait_stream(side)
        self.state.copy_(saved)
        del saved
        torch.cuda.synchronize(self.state.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="relaxed"):
            s = torch.cuda.current_stream()
            self.advance(bg, tau_i, t0, dt, nsteps, s)
            if diagnostics:
                self.diagnostics_async(bg, tau_i + t0 + nsteps * dt, per_cell_fp32=per_cell_fp32, stream=s)
        return g

    def autotune(self, bg: Background, tau_i: float, dt: float, steps: int = 4, repeats: int = 2,
                 z_chunks=(0, 8, 16, 32, 64)) -> dict:
        """Time every compiled tiling x z-chunk target on these boxes and keep the
        fastest (tilings that do not suit every box are left out). The state is
        saved and restored. `steps` is rounded up to an even count: the fused
        step copies the state once on an odd count. Returns {"name zN": ms/step}."""
        steps += steps & 1
        saved = self.state.clone()
        timings = {}
        best = (float("inf"), self.plan.tile_config, self.plan.z_chunk)
        for cid, name in self.tile_configs():
            for zc in z_chunks:
                try:
                    self.init(cid, zc)
                except L.AxsError as err:
                    if err.status != L.AXS_ERR_UNSUPPORTED:
                        raise
                    break
                self.advance(bg, tau_i, 0.0, dt, 1)
                ms = float("inf")
                for _ in range(repeats):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    self.advance(bg, tau_i, 0.0, dt, steps)
                    e1.record()
                    e1.synchronize()
                    ms = min(ms, e0.elapsed_time(e1) / steps)
                timings[f"{name} z{zc if zc else 'auto'}"] = ms
                if ms < best[0]:
                    best = (ms, cid, zc)
        self.init(best[1], best[2])
        self.state.copy_(saved)
        self.device_status()
        return timings
