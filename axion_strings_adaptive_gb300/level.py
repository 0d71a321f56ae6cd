"""Host-side mirror of the reference's per-level interface over the C ABI.

* :func:`fab` / :class:`FabTensor` -- an AMReX FArrayBox held in a torch CUDA
  tensor of shape (ncomp, nz+2ng, ny+2ng, nx+2ng), passed to the library as a
  plain ``axs_fab`` descriptor.
* :class:`PeriodicLevel` -- a single-box periodic level in the fused-RK4
  device layout, with the classic-RK4 advance and the fused diagnostics pass.
* :class:`AxionStringsLevel` -- the GRTeclyn level hooks the reference
  overrides (AxionStrings/AxionStringsLevel.hpp:18-46): ``specific_eval_rhs``
  (per-stage RHS on FABs), ``advance`` (the RK4 level step) and
  ``specific_post_timestep`` (string count, xi, energies, velocities).

torch supplies device memory and streams only; every computation runs in
libaxs_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import torch

from . import _lib as L
from .background import Background, xi_from_comoving_length

_DT = {torch.float32: L.AXS_F32, torch.float64: L.AXS_F64}


def _stream_ptr(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


def _require_cuda(t: torch.Tensor, name: str) -> None:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (the hot path has no CPU implementation)")
    if t.dtype not in _DT:
        raise TypeError(f"{name}: dtype must be float32 or float64, got {t.dtype}")


# ----------------------------------------------------------------------- FABs
def fab(t: torch.Tensor, ng: int) -> L.Fab:
    """Descriptor of a FAB tensor (ncomp, nz+2ng, ny+2ng, nx+2ng), x fastest."""
    _require_cuda(t, "fab")
    if t.dim() != 4:
        raise ValueError("FAB tensors are (ncomp, z, y, x)")
    if t.stride(3) != 1:
        raise ValueError("FAB tensors need unit x stride")
    nc, gz, gy, gx = t.shape
    return L.Fab(t.data_ptr(), _DT[t.dtype], gx - 2 * ng, gy - 2 * ng, gz - 2 * ng, ng, nc, t.stride(2), t.stride(1),
                 t.stride(0))


def new_fab(n, ng: int, dtype=torch.float64, ncomp: int = 4, device="cuda") -> torch.Tensor:
    nx, ny, nz = n
    return torch.zeros((ncomp, nz + 2 * ng, ny + 2 * ng, nx + 2 * ng), dtype=dtype, device=device)


def valid(t: torch.Tensor, ng: int) -> torch.Tensor:
    """The valid-cell view (ncomp, nz, ny, nx) of a FAB tensor."""
    if ng == 0:
        return t
    return t[:, ng:-ng, ng:-ng, ng:-ng]


def eval_rhs(soln: torch.Tensor, rhs: torch.Tensor, ng_soln: int, ng_rhs: int, dx: float, coeffs: L.RhsCoeffs,
             stream=None) -> None:
    L.call("axs_eval_rhs", C.byref(fab(soln, ng_soln)), C.byref(fab(rhs, ng_rhs)), float(dx), C.byref(coeffs),
           _stream_ptr(stream))


def fill_periodic_ghosts(t: torch.Tensor, ng: int, stream=None) -> None:
    L.call("axs_fill_periodic_ghosts", C.byref(fab(t, ng)), _stream_ptr(stream))


def lincomb(dst, x, b: float, y, ng: int, stream=None) -> None:
    L.call("axs_lincomb", C.byref(fab(dst, ng)), C.byref(fab(x, ng)), float(b), C.byref(fab(y, ng)),
           _stream_ptr(stream))


def rk4_combine(dst, uold, k1, k2, k3, k4, ng: int, dt: float, stream=None) -> None:
    L.call("axs_rk4_combine", *[C.byref(fab(t, ng)) for t in (dst, uold, k1, k2, k3, k4)], float(dt),
           _stream_ptr(stream))


# ----------------------------------------------------------------------- diagnostics
ENERGY_FIELDS = ("rho_tot", "rho_axion_kinetic", "rho_axion_gradient", "rho_radial_kinetic",
                 "rho_radial_gradient", "rho_radial_mass")


@dataclass
class Diagnostics:
    """specific_post_timestep's single-level quantities (AxionStringsLevel.cpp:1256-1434)."""
    n_p_plain: int
    n_p_weighted: int
    xi_plain: float
    xi_weighted: float
    energy: dict            # TotalEnergyResult fields (EnergyKernel.hpp:42-75), volumes in n_total/n_unmasked
    energy_sums: list       # the 14 raw sums, EnergyKernel.hpp:196-199 order
    vel_sum: float
    vel_count: int
    mean_gamma_sq_v_sq: float
    mean_gamma: float
    tension_core_only: float
    tension_core_plus_tail: float
    n_near_tie: int
    n_listed: int
    pierced: torch.Tensor | None = field(default=None, repr=False)


def _result_from_bytes(buf: torch.Tensor) -> L.DiagResult:
    host = buf.cpu().numpy().tobytes()
    return L.DiagResult.from_buffer_copy(host)


def summarise(r: L.DiagResult, *, n_cells: int, dx: float, L_tilde: float, a_inv: float, tau: float,
              R: float, pierced: torch.Tensor | None = None) -> Diagnostics:
    s = list(r.energy_sums)
    vol = dx ** 3
    n_total = n_cells * vol
    n_unmasked = s[12] * vol
    energy = {"n_total": n_total, "n_unmasked": n_unmasked}
    for q, name in enumerate(ENERGY_FIELDS):
        energy[name + "_unscreened"] = s[2 * q] / n_cells
        energy[name + "_screened"] = s[2 * q + 1] / s[12] if s[12] > 0.0 else 0.0
    ell_plain = (2.0 / 3.0) * r.n_p_plain * dx
    ell_weighted = (2.0 / 3.0) * r.n_p_weighted * dx
    mean_g = r.vel_sum / r.vel_count if r.vel_count > 0 else 0.0
    core = n_total * energy["rho_tot_unscreened"] - n_unmasked * energy["rho_tot_screened"]
    tail = n_unmasked * (energy["rho_axion_gradient_screened"] - energy["rho_axion_kinetic_screened"])
    t_core = (R * R) * core / ell_plain if ell_plain > 0.0 else 0.0
    t_tail = (R * R) * (core + tail) / ell_plain if ell_plain > 0.0 else 0.0
    return Diagnostics(r.n_p_plain, r.n_p_weighted, xi_from_comoving_length(ell_plain, L_tilde, a_inv, tau),
                       xi_from_comoving_length(ell_weighted, L_tilde, a_inv, tau), energy, s, r.vel_sum,
                       r.vel_count, mean_g, math.sqrt(1.0 + mean_g), t_core, t_tail, r.n_near_tie, r.n_listed,
                       pierced)


def scratch_bytes(nx: int, ny: int, nz: int) -> int:
    b = C.c_int64()
    L.call("axs_diagnostics_scratch_bytes", nx, ny, nz, C.byref(b))
    return b.value


# ----------------------------------------------------------------------- periodic level
class PeriodicLevel:
    """One periodic box in the fused-RK4 layout (see axs_level_layout in include/axs.h).

    ``state`` is (4, nz, ny+4, jstride); the valid cells are
    ``state[:, :, y_offset:y_offset+ny, x_offset:x_offset+nx]``, with x = 0 on a
    128-byte boundary. ``work`` holds the 8 between-sweep components and the
    device status word.
    """

    def __init__(self, n, dx: float, dtype=torch.float32, device="cuda", pierced_capacity: int | None = None,
                 tile_config: int = 0):
        nx, ny, nz = (n, n, n) if isinstance(n, int) else n
        self.nx, self.ny, self.nz, self.dx, self.dtype = nx, ny, nz, float(dx), dtype
        lay = L.LevelLayout()
        L.call("axs_level_layout_for", _DT[dtype], nx, ny, nz, C.byref(lay))
        self.layout = lay
        es = torch.finfo(dtype).bits // 8
        self.state = torch.zeros((4, nz, ny + 4, lay.jstride), dtype=dtype, device=device)
        assert self.state.numel() * es == lay.state_bytes
        self.work = torch.zeros(lay.work_bytes, dtype=torch.uint8, device=device)
        self.c = L.LevelC(self.state.data_ptr(), self.work.data_ptr(), _DT[dtype], nx, ny, nz, self.dx,
                          int(tile_config))
        # diagnostics buffers (allocated once; the pass itself allocates nothing)
        self._scratch = torch.zeros(scratch_bytes(nx, ny, nz), dtype=torch.uint8, device=device)
        self._result = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device=device)
        cap = pierced_capacity if pierced_capacity is not None else max(1024, 3 * nx * ny * nz // 16)
        self._pierced = torch.zeros(cap, dtype=torch.int64, device=device)

    @property
    def n_cells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def L_tilde(self) -> float:
        return self.nx * self.dx

    def valid_view(self) -> torch.Tensor:
        ox, oy = self.layout.x_offset, self.layout.y_offset
        return self.state[:, :, oy:oy + self.ny, ox:ox + self.nx]

    @property
    def tile_config(self) -> int:
        return self.c.tile_config

    @tile_config.setter
    def tile_config(self, v: int) -> None:
        self.c.tile_config = int(v)

    @property
    def compensated(self) -> bool:
        """FP32 steps with the FP32 remainders of the Laplacian weights and the
        step fractions applied (AXS_LEVEL_COMPENSATED_FP32; no effect in FP64)."""
        return bool(self.c.flags & L.LEVEL_COMPENSATED_FP32)

    @compensated.setter
    def compensated(self, on: bool) -> None:
        self.c.flags = (self.c.flags | L.LEVEL_COMPENSATED_FP32) if on else (self.c.flags & ~L.LEVEL_COMPENSATED_FP32)

    def tile_configs(self) -> list:
        """(id, name) of every sweep tiling compiled for this level's dtype."""
        lib = L.lib()
        d = _DT[self.dtype]
        return [(i, lib.axs_level_tile_config_name(d, i).decode()) for i in range(1, lib.axs_level_tile_config_count(d) + 1)]

    def autotune(self, bg: Background, tau_i: float, dt: float, steps: int = 4, repeats: int = 2,
                 stream=None) -> dict:
        """Time every compiled tiling on this level (the two-sweep tilings and
        the one-pass fused step; full RK4 steps, CUDA events) and keep the
        fastest. An even step count times the fused step alone (an odd count
        runs its first step as the two sweeps). The state is saved and restored, so the
        level's contents are unchanged. Returns {name: ms_per_step}."""
        saved = self.state.clone()
        timings = {}
        best = (float("inf"), self.c.tile_config)
        for cid, name in self.tile_configs():
            self.c.tile_config = cid
            self.advance(bg, tau_i, 0.0, dt, 1, stream)  # warm-up (sets up the kernel)
            ms = float("inf")
            for _ in range(repeats):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self.advance(bg, tau_i, 0.0, dt, steps, stream)
                e1.record()
                e1.synchronize()
                ms = min(ms, e0.elapsed_time(e1) / steps)
            timings[name] = ms
            if ms < best[0]:
                best = (ms, cid)
        self.c.tile_config = best[1]
        self.state.copy_(saved)
        self.device_status(stream)
        return timings

    def set_state(self, valid_cells: torch.Tensor, stream=None) -> None:
        """Copy (4, nz, ny, nx) valid cells in and refresh the periodic padding."""
        self.valid_view().copy_(valid_cells.to(device=self.state.device, dtype=self.dtype))
        L.call("axs_level_fill_ghosts", C.byref(self.c), _stream_ptr(stream))

    def get_state(self) -> torch.Tensor:
        return self.valid_view().clone()

    def import_fab(self, t: torch.Tensor, ng: int, stream=None) -> None:
        L.call("axs_level_import_fab", C.byref(self.c), C.byref(fab(t, ng)), _stream_ptr(stream))

    def export_fab(self, t: torch.Tensor, ng: int, stream=None) -> None:
        L.call("axs_level_export_fab", C.byref(self.c), C.byref(fab(t, ng)), _stream_ptr(stream))

    def advance(self, bg: Background, tau_i: float, t0: float, dt: float, nsteps: int, stream=None) -> None:
        """nsteps classic-RK4 steps (two fused sweeps each); asynchronous."""
        L.call("axs_level_rk4_advance", C.byref(self.c), C.byref(bg.to_c()), float(tau_i), float(t0), float(dt),
               int(nsteps), _stream_ptr(stream))

    def step_to(self, dst: torch.Tensor, bg: Background, tau_i: float, t: float, dt: float, stream=None) -> None:
        """One RK4 step from t written into `dst` (a tensor like ``state``); the
        level's state is unchanged (axs_level_rk4_step_to); asynchronous."""
        if dst.shape != self.state.shape or dst.dtype != self.dtype or dst.device != self.state.device or \
                not dst.is_contiguous():
            raise ValueError("step_to needs a contiguous tensor of the state's shape, dtype and device")
        L.call("axs_level_rk4_step_to", C.byref(self.c), dst.data_ptr(), C.byref(bg.to_c()), float(tau_i), float(t),
               float(dt), _stream_ptr(stream))

    def swap_state(self, other: torch.Tensor) -> torch.Tensor:
        """Make `other` (a tensor like ``state``) the level's state and return the
        previous state tensor; no data moves."""
        if other.shape != self.state.shape or other.dtype != self.dtype or other.device != self.state.device or \
                not other.is_contiguous():
            raise ValueError("swap_state needs a contiguous tensor of the state's shape, dtype and device")
        old, self.state = self.state, other
        self.c.state = self.state.data_ptr()
        return old

    def sweep(self, bg: Background, tau_i: float, t: float, dt: float, which: int, stream=None) -> None:
        """Sweep A (0) or B (1) of the step starting at t; A then B is one RK4 step."""
        L.call("axs_level_rk4_sweep", C.byref(self.c), C.byref(bg.to_c()), float(tau_i), float(t), float(dt),
               int(which), _stream_ptr(stream))

    def device_status(self, stream=None) -> None:
        L.call("axs_level_device_status", C.byref(self.c), _stream_ptr(stream))

    def count_nonfinite(self, stream=None) -> int:
        """Valid cells with a NaN or infinite component (axs_level_count_nonfinite);
        synchronises the stream to read the count."""
        if getattr(self, "_nonfinite", None) is None:
            self._nonfinite = torch.zeros(1, dtype=torch.int64, device=self.state.device)
        L.call("axs_level_count_nonfinite", C.byref(self.c), self._nonfinite.data_ptr(), _stream_ptr(stream))
        return int(self._nonfinite.item())

    def tag_cells(self, gradient_threshold: float = 1.7976931348623157e308,
                  radial_gradient_threshold: float = 1.7976931348623157e308, n_error_buf: int = 0,
                  block: int = 0, stream=None):
        """AxionStringsLevel::tag_cells' criterion (StringTagger) plus the
        n_error_buf cube buffer. Returns (tags (nz, ny, nx) uint8 CUDA tensor,
        n_tagged, block flags (nbz, nby, nbx) or None)."""
        nx, ny, nz = self.nx, self.ny, self.nz
        dev = self.state.device
        if getattr(self, "_tag_scratch", None) is None:
            b = C.c_int64()
            L.call("axs_tag_scratch_bytes", nx, ny, nz, C.byref(b))
            self._tag_scratch = torch.zeros(b.value, dtype=torch.uint8, device=dev)
            self._n_tagged = torch.zeros(1, dtype=torch.int64, device=dev)
        tags = torch.empty((nz, ny, nx), dtype=torch.uint8, device=dev)
        flags = None
        if block > 0:
            flags = torch.empty((-(-nz // block), -(-ny // block), -(-nx // block)), dtype=torch.uint8, device=dev)
        p = L.TagParams(self.dx, float(gradient_threshold), float(radial_gradient_threshold), int(n_error_buf),
                        int(block))
        L.call("axs_level_tag_cells", C.byref(self.c), C.byref(p), tags.data_ptr(),
               flags.data_ptr() if flags is not None else None, self._n_tagged.data_ptr(),
               self._tag_scratch.data_ptr(), self._tag_scratch.numel(), _stream_ptr(stream))
        return tags, int(self._n_tagged.item()), flags

    def diagnostics_raw(self, params: L.DiagParams, mask: torch.Tensor | None = None, want_list: bool = True,
                        stream=None) -> L.DiagResult:
        mptr = None
        if mask is not None:
            if mask.dtype != torch.uint8 or not mask.is_cuda or mask.numel() != self.n_cells:
                raise ValueError("mask must be a CUDA uint8 tensor with one entry per valid cell")
            mptr = mask.data_ptr()
        cap = self._pierced.numel() if want_list else 0
        L.call("axs_level_diagnostics", C.byref(self.c), C.byref(params), mptr, self._result.data_ptr(),
               self._pierced.data_ptr() if want_list else None, cap, self._scratch.data_ptr(),
               self._scratch.numel(), _stream_ptr(stream))
        torch.cuda.synchronize(self.state.device)
        return _result_from_bytes(self._result)

    def diagnostics(self, bg: Background, tau: float, masking_scheme: int = L.MASK_A, threshold: float = 0.8,
                    mask: torch.Tensor | None = None, want_list: bool = True, per_cell_fp32: bool = False,
                    strings_only: bool = False, stream=None) -> Diagnostics:
        """specific_post_timestep's pass. per_cell_fp32 (FP32 levels): per-cell
        terms in FP32 with FP64 accumulation instead of the reference's double
        per-cell arithmetic (energies to ~1e-7 relative, counts exact).
        strings_only: the string finder alone (count_plaquettes and the pierced
        list; energies and the velocity are left at zero)."""
        v = bg.values(tau)
        rpr = 0.0 if bg.kind == L.BG_FLAT else v.R_prime_over_R
        want = (0, 1, 0) if strings_only else (1, 1, 1)
        p = L.DiagParams(self.dx, v.R, v.lambda_, rpr, v.m_r, masking_scheme, threshold, L.BOUNDARY_PERIODIC, *want,
                         int(per_cell_fp32))
        r = self.diagnostics_raw(p, mask, want_list, stream)
        if r.status == L.AXS_ERR_CAPACITY:
            raise L.AxsError(L.AXS_ERR_CAPACITY, "pierced-plaquette list capacity exceeded")
        pierced = self._pierced[: r.n_listed].clone() if want_list else None
        return summarise(r, n_cells=self.n_cells, dx=self.dx, L_tilde=self.L_tilde, a_inv=bg.a_inv, tau=tau, R=v.R,
                         pierced=pierced)


# ----------------------------------------------------------------------- level hooks
class AxionStringsLevel:
    """The reference level's hot-path hooks (AxionStringsLevel.hpp:18-46) over the C ABI.

    Conformal time is ``tau = tau_i + a_time`` as in the reference
    (AxionStringsLevel.hpp:65-72).
    """

    def __init__(self, n, dx: float, background: Background, tau_i: float = 1.0, dtype=torch.float32,
                 masking_scheme: int = L.MASK_A, masking_threshold: float = 0.8, device="cuda",
                 compensated: bool = False):
        """compensated: the compensated FP32 step (PeriodicLevel.compensated)."""
        self.bg = background
        self.tau_i = float(tau_i)
        self.time = 0.0
        self.masking_scheme = masking_scheme
        self.masking_threshold = masking_threshold
        self.level = PeriodicLevel(n, dx, dtype=dtype, device=device)
        self.level.compensated = compensated

    @property
    def tau(self) -> float:
        return self.tau_i + self.time

    # AxionStringsLevel::specific_eval_rhs (AxionStringsLevel.cpp:850-921)
    def specific_eval_rhs(self, soln: torch.Tensor, rhs: torch.Tensor, a_time: float, ng_soln: int = 2,
                          ng_rhs: int = 0, stream=None) -> None:
        eval_rhs(soln, rhs, ng_soln, ng_rhs, self.level.dx, self.bg.rhs_coeffs(self.tau_i + a_time), stream)

    # GRTeclyn's RK4 level advance (fused two-sweep kernels)
    def advance(self, dt: float, nsteps: int = 1, stream=None) -> None:
        self.level.advance(self.bg, self.tau_i, self.time, dt, nsteps, stream)
        self.time += nsteps * dt

    # AxionStringsLevel::apply_pre_evolution_to_main_rescale (AxionStringsLevel.cpp:2027-2132)
    def apply_pre_evolution_to_main_rescale(self, main_background: Background, tau_i_main: float,
                                            transition_n_periods: float = 0.0, stream=None) -> None:
        """End pre-evolution: this level has run on its pre-evolution background
        with the pre-evolution clock (tau = time, tau_i = 0). Rescale psi, Pi onto
        the main background at tau_i_main, switch to it, and shift tau_i so that
        tau = tau_i + time equals tau_i_main now. With transition_n_periods > 0,
        lambda and the curvature coefficient blend from their frozen
        pre-evolution values over that many main-schedule core periods."""
        import dataclasses
        import math
        pre = self.bg
        tau_pre_end = self.time
        vp, vm = pre.values(tau_pre_end), main_background.values(tau_i_main)
        L.call("axs_level_handoff_rescale", C.byref(self.level.c), vp.R, vp.R_prime, vm.R, vm.R_prime,
               _stream_ptr(stream))
        bg = main_background
        if transition_n_periods > 0.0:
            lam_start = vp.lambda_
            lam_main = vm.lambda_
            m_r_period = math.sqrt(lam_main) if lam_main > 0.0 else math.sqrt(lam_start)
            bg = dataclasses.replace(main_background, blend_dtau=transition_n_periods * 2.0 * math.pi / m_r_period,
                                     blend_tau_start=tau_i_main, blend_lambda_start=lam_start,
                                     blend_curv_start=vp.kappa)
        self.bg = bg
        self.tau_i = tau_i_main - tau_pre_end

    def check_finite(self, stream=None) -> None:
        """Raise FloatingPointError if any valid cell holds a NaN or infinite
        component (a run that has blown up). The reference has no such check."""
        n = self.level.count_nonfinite(stream)
        if n:
            raise FloatingPointError(f"{n} cells of the level hold NaN or infinite values at tau = {self.tau}")

    # AxionStringsLevel::specific_post_timestep's diagnostics (AxionStringsLevel.cpp:1256-1434)
    def specific_post_timestep(self, mask: torch.Tensor | None = None, want_list: bool = True) -> Diagnostics:
        return self.level.diagnostics(self.bg, self.tau, self.masking_scheme, self.masking_threshold, mask,
                                      want_list)
