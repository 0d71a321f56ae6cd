"""Two-level block-structured refinement on a periodic coarse level (the scale path).

The coarse level is a :class:`~.level.PeriodicLevel`. The refinement tagger
(``axs_level_tag_cells``: the StringTagger criteria plus an ``n_error_buf``
buffer) flags block^3 blocks of coarse cells; every flagged block gets a patch
of (2 block)^3 fine cells (:class:`Patches`, ``axs_patches_*``). One coarse
step advances the coarse level by dt and then the patches by two fine steps of
dt/2 (subcycling), each after refilling the patch ghost rings from neighbouring
patches or, where none owns a ring cell, from the coarse level interpolated in
space and time. As in the reference, the coarse level keeps evolving under the
patches (nothing averages fine data down during the evolution);
:meth:`TwoLevel.collapse_to_coarse` averages down on request, e.g. before a
spectrum. :meth:`TwoLevel.diagnostics` is the composite of
specific_post_timestep (AxionStringsLevel.cpp:1296-1350): the coarse level
with its covered cells masked out plus every patch, string lengths weighted by
dx, velocities by dx, energies by dx^3 (EnergyKernel.hpp:287-339).
"""
from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np
import torch

from . import _lib as L
from .background import Background, xi_from_comoving_length
from .level import _DT, PeriodicLevel, _stream_ptr


class Patches:
    """npatches refined patches of n^3 fine cells (spacing dx) with ghost rings."""

    def __init__(self, n: int, npatches: int, dx: float, dtype=torch.float32, device="cuda",
                 storage: torch.Tensor | None = None, clear: bool = True, capacity: int | None = None):
        """capacity: patch slots the arena's component planes are laid out for
        (>= npatches; default npatches): a later patch set of up to that many
        patches can live in the same arena with every kept patch in place.
        storage: a 1-D tensor of dtype to lay the state arena in (its first
        4 plane_elems elements), when it is large enough; else a new one.
        clear: zero the arena (a caller that writes every box itself skips it)."""
        cap = int(npatches) if capacity is None else max(int(capacity), int(npatches))
        lay = L.PatchLayout()
        L.call("axs_patches_layout", _DT[dtype], int(n), cap, C.byref(lay))
        lay_n = L.PatchLayout()
        L.call("axs_patches_layout", _DT[dtype], int(n), int(npatches), C.byref(lay_n))
        self.layout, self.n, self.npatches, self.capacity = lay, int(n), int(npatches), cap
        self.dx, self.dtype = float(dx), dtype
        need = 4 * lay.plane_elems
        if storage is None or storage.dtype != dtype or storage.numel() < need:
            storage = torch.empty(need, dtype=dtype, device=device)
        self.storage = storage
        self.state = storage[:need].view(4, lay.plane_elems)
        if clear:
            self.state.zero_()
        # sweep A writes every work cell sweep B reads, so the work planes need no
        # clearing; patch sizes the fused step covers need no work arena
        self.work = torch.empty((8, lay.plane_elems) if lay.work_bytes > 0 else (0,), dtype=dtype, device=device)
        self.table = torch.zeros(lay_n.table_bytes, dtype=torch.uint8, device=device)
        self.c = L.PatchesC(_DT[dtype], self.n, self.npatches, self.dx, self.state.data_ptr(), self.work.data_ptr(),
                            self.table.data_ptr(), lay.state_bytes, lay.work_bytes, lay_n.table_bytes, cap)
        self.plan = L.PatchPlan()
        L.call("axs_patches_init", C.byref(self.c), C.byref(self.plan), None)

    def box(self, q: int, arena: torch.Tensor | None = None) -> torch.Tensor:
        """(ncomp, n+8, n+8, jstride) padded box of patch q."""
        t = self.state if arena is None else arena
        lay, n = self.layout, self.n
        blk = t[:, q * lay.patch_elems:q * lay.patch_elems + (n + 8) * lay.kstride]
        return blk.view(t.shape[0], n + 8, n + 8, lay.jstride)

    def valid(self, q: int, arena: torch.Tensor | None = None) -> torch.Tensor:
        lay, n = self.layout, self.n
        return self.box(q, arena)[:, lay.z_offset:lay.z_offset + n, lay.y_offset:lay.y_offset + n,
                                  lay.x_offset:lay.x_offset + n]

    def step(self, bg: Background, tau_i: float, t: float, dt: float, stream=None) -> None:
        L.call("axs_patches_rk4_step", C.byref(self.c), C.byref(self.plan), C.byref(bg.to_c()), float(tau_i),
               float(t), float(dt), _stream_ptr(stream))

    def device_status(self) -> None:
        L.call("axs_patches_device_status", C.byref(self.c), None)

    def diagnostics(self, prm: L.DiagParams, list_capacity: int = 0):
        """One diagnostics pass over every patch (rings as ghost cells), summed
        into one DiagResult; with list_capacity > 0 also the pierced list
        (entries 4 (q n^3 + cell) + plane), returned as (result, list)."""
        nbytes = C.c_int64()
        L.call("axs_patches_diagnostics_scratch_bytes", self.n, self.npatches, C.byref(nbytes))
        dev = self.state.device
        scratch = torch.zeros(nbytes.value, dtype=torch.uint8, device=dev)
        res = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device=dev)
        lst = torch.zeros(max(1, list_capacity), dtype=torch.int64, device=dev)
        L.call("axs_patches_diagnostics", C.byref(self.c), C.byref(prm), res.data_ptr(),
               lst.data_ptr() if list_capacity > 0 else None, int(list_capacity), scratch.data_ptr(), scratch.numel(),
               torch.cuda.current_stream().cuda_stream)
        out = L.DiagResult.from_buffer_copy(res.cpu().numpy().tobytes())
        L.check(out.status)
        if list_capacity > 0:
            return out, lst[:out.n_listed].clone()
        return out

    def fab(self, q: int) -> L.Fab:
        """axs_fab view of patch q with 4 ghost layers (its ring), for the diagnostics pass."""
        lay, es = self.layout, torch.finfo(self.dtype).bits // 8
        ptr = self.state.data_ptr() + (q * lay.patch_elems + lay.x_offset - 4) * es
        return L.Fab(ptr, _DT[self.dtype], self.n, self.n, self.n, 4, 4, lay.jstride, lay.kstride, lay.plane_elems)


@dataclasses.dataclass
class CompositeDiagnostics:
    n_p_plain: int
    n_p_weighted: int
    xi_plain: float
    xi_weighted: float
    energy: dict
    mean_gamma_sq_v_sq: float
    vel_count: int
    n_patches: int
    refined_fraction: float


def in_place_slots(old_q: np.ndarray, n_new: int):
    """The slot plan of a regrid inside the same arena.

    old_q[i] is the patch slot that block i of the new set held before (-1: the
    block is newly refined). Kept patches whose slot lies below n_new stay
    there; kept patches at or above n_new move into the free slots below it, in
    order; new patches take the slots left. Returns (slot of each block,
    src_of_dst per slot for axs_patches_copy_boxes: PATCH_KEEP where the patch
    stays, the old slot it is copied from, or -1 for a new patch, and the slots
    of the new patches)."""
    old_q = np.asarray(old_q, dtype=np.int64)
    slot = np.full(n_new, -1, dtype=np.int64)
    stay = (old_q >= 0) & (old_q < n_new)
    slot[stay] = old_q[stay]
    used = np.zeros(n_new, dtype=bool)
    used[old_q[stay]] = True
    holes = np.nonzero(~used)[0]
    movers = np.nonzero(old_q >= n_new)[0]
    fresh = np.nonzero(old_q < 0)[0]
    slot[movers] = holes[:len(movers)]
    slot[fresh] = holes[len(movers):]
    src_of_dst = np.full(n_new, L.PATCH_KEEP, dtype=np.int32)
    src_of_dst[slot[movers]] = old_q[movers]
    src_of_dst[slot[fresh]] = -1
    return slot, src_of_dst, slot[fresh].astype(np.int32)


class TwoLevel:
    """A periodic coarse level plus 2x-refined patches on tagged block^3 blocks."""

    ENERGY_NAMES = ["rho_tot", "rho_axion_kinetic", "rho_axion_gradient", "rho_radial_kinetic",
                    "rho_radial_gradient", "rho_radial_mass"]

    def __init__(self, coarse: PeriodicLevel, block: int = 32, headroom: float = 1.25):
        """headroom: the patch arena is laid out for headroom x the patch count
        (patch slots), so that regrids whose patch count stays within that keep
        one arena: kept patches stay in their slots (or move down into free ones),
        new patches take free slots. A regrid past the capacity lays the patches
        out in a new arena once."""
        if coarse.nx % block or coarse.ny % block or coarse.nz % block:
            raise ValueError("the coarse level must tile into blocks")
        self.coarse, self.block = coarse, int(block)
        self.headroom = float(headroom)
        self.nb = (coarse.nx // block, coarse.ny // block, coarse.nz // block)
        # the coarse state at the start of the running coarse step (state only: the
        # ghost fill reads nothing else)
        self.old_state = torch.zeros_like(coarse.state)
        self.old_c = L.LevelC(self.old_state.data_ptr(), coarse.work.data_ptr(), coarse.c.dtype, coarse.nx, coarse.ny,
                              coarse.nz, coarse.dx, 0)
        self.patches: Patches | None = None
        self.blocks = np.zeros((0, 3), dtype=np.int32)
        dev = coarse.state.device
        # block -> patch slot (-1: not refined), on the device for the kernels and
        # on the host for the regrid's bookkeeping
        self._block_patch_host = np.full((self.nb[2], self.nb[1], self.nb[0]), -1, dtype=np.int32)
        self._block_patch = torch.from_numpy(self._block_patch_host.copy()).to(dev)
        self._patch_block = torch.zeros((1, 3), dtype=torch.int32, device=dev)

    # ------------------------------------------------------------------ patch management
    def _map(self) -> L.PatchMap:
        return L.PatchMap(self._patch_block.data_ptr(), self._block_patch.data_ptr())

    def set_blocks(self, blocks: np.ndarray) -> None:
        """Refine exactly these blocks ((k, 3) block coordinates x, y, z): blocks
        refined before keep their fine data, new ones interpolate the coarse level.

        Within the arena's capacity the new set is laid out in the same arena: a
        kept patch whose slot lies below the new patch count stays where it is,
        kept patches above it move into the free slots below it, and new patches
        take the slots left (one box-copy launch moves and clears, one fill
        interpolates the new patches). Past the capacity, a new arena of headroom
        x the count receives the kept patches."""
        blocks = np.asarray(blocks, dtype=np.int32).reshape(-1, 3)
        dev = self.coarse.state.device
        old_patches = self.patches
        n_new = len(blocks)
        if n_new == 0:
            self.blocks = blocks
            self.patches = None
            self._block_patch.fill_(-1)
            self._block_patch_host.fill(-1)
            return
        dt = self.coarse.dtype
        if old_patches is not None:
            old_q = self._block_patch_host[blocks[:, 2], blocks[:, 1], blocks[:, 0]].astype(np.int64)
        else:
            old_q = np.full(n_new, -1, dtype=np.int64)
        in_place = old_patches is not None and n_new <= old_patches.capacity
        if in_place:
            slot, src_of_dst, new_slots = in_place_slots(old_q, n_new)
            order = np.argsort(slot)  # patch q holds block order[q]
            blocks = blocks[order]
            storage, cap = old_patches.storage, old_patches.capacity
        else:
            src_of_dst = old_q.astype(np.int32)  # -1: newly refined (cleared, then interpolated)
            new_slots = np.nonzero(old_q < 0)[0].astype(np.int32)
            # a new arena; the old one is read by the copy below and then released
            # (stream-ordered: the allocator reuses it only after that copy)
            storage, cap = None, max(n_new, int(np.ceil(n_new * self.headroom)))
        self.blocks = blocks
        self.patches = Patches(2 * self.block, n_new, 0.5 * self.coarse.dx, dtype=dt, device=dev, storage=storage,
                               clear=False, capacity=cap)
        self._patch_block = torch.from_numpy(blocks.copy()).to(dev)
        bp = np.full((self.nb[2], self.nb[1], self.nb[0]), -1, dtype=np.int32)
        bp[blocks[:, 2], blocks[:, 1], blocks[:, 0]] = np.arange(n_new, dtype=np.int32)
        self._block_patch_host = bp
        self._block_patch = torch.from_numpy(bp.copy()).to(dev)
        sod = torch.from_numpy(src_of_dst).to(dev)
        # whole patch boxes (valid cells and rings; the rings are refilled before use)
        L.call("axs_patches_copy_boxes", C.byref(self.patches.c),
               C.byref(old_patches.c) if old_patches is not None else None, sod.data_ptr(), None)
        if len(new_slots):
            lst = torch.from_numpy(new_slots).to(dev)
            L.call("axs_patches_fill_list", C.byref(self.patches.c), C.byref(self._map()), C.byref(self.coarse.c),
                   None, 0.0, 0.0, 1, lst.data_ptr(), int(lst.numel()), None)

    def regrid(self, n_error_buf: int = 4, gradient_threshold: float = 1.7976931348623157e308,
               radial_gradient_threshold: float = 1.7976931348623157e308) -> int:
        """Tag the coarse level (StringTagger + buffer) and refine every block holding a tag."""
        _, _, flags = self.coarse.tag_cells(gradient_threshold, radial_gradient_threshold, n_error_buf, self.block)
        idx = torch.nonzero(flags.cpu()).numpy()  # (bz, by, bx)
        self.set_blocks(idx[:, ::-1].astype(np.int32))
        return len(idx)

    # ------------------------------------------------------------------ evolution
    def advance(self, bg: Background, tau_i: float, t0: float, dt: float, nsteps: int) -> None:
        """nsteps coarse steps, each followed by two subcycled fine steps."""
        for s in range(nsteps):
            t = t0 + s * dt
            if self.patches is None:
                self.coarse.advance(bg, tau_i, t, dt, 1)
                continue
            # the step goes into the spare buffer, which then becomes the state;
            # the previous state stays in the other one as the step's start
            self.coarse.step_to(self.old_state, bg, tau_i, t, dt)
            self.old_state = self.coarse.swap_state(self.old_state)
            self.old_c.state = self.old_state.data_ptr()
            for f, theta in enumerate((0.0, 0.5)):
                L.call("axs_patches_fill", C.byref(self.patches.c), C.byref(self._map()), C.byref(self.old_c),
                       C.byref(self.coarse.c), theta, dt, 0, None)
                self.patches.step(bg, tau_i, t + f * 0.5 * dt, 0.5 * dt)

    def device_status(self) -> None:
        self.coarse.device_status()
        if self.patches is not None:
            self.patches.device_status()

    def collapse_to_coarse(self) -> None:
        """amrex::average_down of every patch onto the coarse level (in place)."""
        if self.patches is not None:
            L.call("axs_patches_average_down", C.byref(self.patches.c), C.byref(self._map()), C.byref(self.coarse.c),
                   None)

    # ------------------------------------------------------------------ composite diagnostics
    def coverage_mask(self) -> torch.Tensor:
        """uint8 (nz, ny, nx) over the coarse cells: 1 where no patch covers the cell."""
        b = self.block
        covered = (self._block_patch >= 0).to(torch.uint8)
        covered = covered.repeat_interleave(b, 0).repeat_interleave(b, 1).repeat_interleave(b, 2)
        return (1 - covered).contiguous()

    def diagnostics(self, bg: Background, tau: float, masking_scheme: int = L.MASK_A, threshold: float = 0.8,
                    strings_only: bool = False, per_cell_fp32: bool = False) -> CompositeDiagnostics:
        """strings_only: the composite count_plaquettes alone (energies and the
        velocity are left at zero); per_cell_fp32: see axs_diag_params."""
        v = bg.values(tau)
        rpr = 0.0 if bg.kind == L.BG_FLAT else v.R_prime_over_R
        want = (0, 1, 0) if strings_only else (1, 1, 1)
        fp32 = int(per_cell_fp32 and self.coarse.dtype == torch.float32)
        levels = []
        mask = self.coverage_mask().reshape(-1) if self.patches is not None else None
        levels.append((self.coarse.diagnostics_raw(
            L.DiagParams(self.coarse.dx, v.R, v.lambda_, rpr, v.m_r, masking_scheme, threshold, L.BOUNDARY_PERIODIC,
                         *want, fp32), mask, want_list=False), self.coarse.dx))
        if self.patches is not None:
            p = self.patches
            # rings at the current time: neighbours, else the (current) coarse level
            L.call("axs_patches_fill", C.byref(p.c), C.byref(self._map()), C.byref(self.coarse.c), None, 0.0, 0.0, 0,
                   None)
            levels.append((p.diagnostics(L.DiagParams(p.dx, v.R, v.lambda_, rpr, v.m_r, masking_scheme, threshold,
                                                      L.BOUNDARY_GHOSTS, *want, fp32)), p.dx))
        # composite combination (AxionStringsLevel.cpp:1302-1350, EnergyKernel.hpp:287-339)
        n_p = sum(r.n_p_plain for r, _ in levels)
        n_w = sum(r.n_p_weighted for r, _ in levels)
        ell_p = sum((2.0 / 3.0) * r.n_p_plain * dx for r, dx in levels)
        ell_w = sum((2.0 / 3.0) * r.n_p_weighted * dx for r, dx in levels)
        vsum = sum(r.vel_sum * dx for r, dx in levels)
        vcnt = sum(r.vel_count * dx for r, dx in levels)
        acc = np.zeros(14)
        for r, dx in levels:
            acc += np.array(list(r.energy_sums)) * dx ** 3
        n_total, n_unmasked = acc[13], acc[12]
        energy = {"n_total": n_total, "n_unmasked": n_unmasked}
        for q, name in enumerate(self.ENERGY_NAMES):
            energy[name + "_unscreened"] = acc[2 * q] / n_total if n_total > 0.0 else 0.0
            energy[name + "_screened"] = acc[2 * q + 1] / n_unmasked if n_unmasked > 0.0 else 0.0
        L_tilde = self.coarse.nx * self.coarse.dx
        nref = 0 if self.patches is None else self.patches.npatches
        return CompositeDiagnostics(
            n_p_plain=n_p, n_p_weighted=n_w, xi_plain=xi_from_comoving_length(ell_p, L_tilde, bg.a_inv, tau),
            xi_weighted=xi_from_comoving_length(ell_w, L_tilde, bg.a_inv, tau), energy=energy,
            mean_gamma_sq_v_sq=vsum / vcnt if vcnt > 0 else 0.0, vel_count=sum(r.vel_count for r, _ in levels),
            n_patches=nref, refined_fraction=nref / float(np.prod(self.nb)))
