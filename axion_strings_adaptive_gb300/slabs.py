"""z-slab decomposition of a periodic box: the halo and reduction seams.

The reference runs one AMReX box layout over MPI ranks: every RK stage's
FillBoundary (AxionStringsLevel.cpp:820, :1255) exchanges ghost cells between
ranks, and every diagnostic is an MPI all-reduce of per-rank sums
(StringFinder.hpp:119-120, EnergyKernel.hpp:215, VelocityKernel.hpp:138-139).
This module is the host side of the same split for the drop-in FAB path, one z
slab per rank:

* :func:`exchange_z_halos` -- x/y ghosts filled periodically on the GPU, the
  edge planes packed by the library, swapped with the neighbouring ranks over
  ``torch.distributed`` (NCCL on GPUs, gloo on CPUs), unpacked into the z ghosts;
* :func:`reduce_diagnostics` -- the all-reduce of the 18 raw scalars of a
  slab's axs_diagnostics result and the exclusive prefix sum that places each
  slab's pierced-plaquette entries in the whole box's numbering.

:func:`exchange_z_halos_local` is the same exchange between slabs held by one
process (tests, single-GPU runs). The device work runs in libaxs_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .level import _stream_ptr, fab


def fill_ghosts_xy(t: torch.Tensor, ng: int, stream=None) -> None:
    L.call("axs_fill_periodic_ghosts_xy", C.byref(fab(t, ng)), _stream_ptr(stream))


def pack_z(t: torch.Tensor, ng: int, side: int, stream=None) -> torch.Tensor:
    """The slab's ng lowest (side 0) or highest (side 1) valid planes, x/y
    ghosts included, as a contiguous (ncomp, ng, ny+2ng, nx+2ng) tensor."""
    nc, gz, gy, gx = t.shape
    nz = gz - 2 * ng
    buf = torch.empty((nc, ng, gy, gx), dtype=t.dtype, device=t.device)
    L.call("axs_fab_pack_z_planes", C.byref(fab(t, ng)), 0 if side == 0 else nz - ng, ng, buf.data_ptr(),
           _stream_ptr(stream))
    return buf


def unpack_z(t: torch.Tensor, ng: int, side: int, buf: torch.Tensor, stream=None) -> None:
    """Planes received from the lower (side 0: into z = -ng .. -1) or upper
    (side 1: into z = nz .. nz+ng-1) neighbour."""
    nz = t.shape[1] - 2 * ng
    L.call("axs_fab_unpack_z_planes", C.byref(fab(t, ng)), -ng if side == 0 else nz, ng, buf.data_ptr(),
           _stream_ptr(stream))


def exchange_z_halos_local(slabs: list, ng: int, stream=None) -> None:
    """Halo exchange between the z slabs of one periodic box held in one
    process (slab s borders s - 1 below and s + 1 above, cyclically)."""
    for t in slabs:
        fill_ghosts_xy(t, ng, stream)
    low = [pack_z(t, ng, 0, stream) for t in slabs]
    high = [pack_z(t, ng, 1, stream) for t in slabs]
    n = len(slabs)
    for s, t in enumerate(slabs):
        unpack_z(t, ng, 0, high[(s - 1) % n], stream)
        unpack_z(t, ng, 1, low[(s + 1) % n], stream)


def exchange_z_halos(t: torch.Tensor, ng: int, group=None, stream=None) -> None:
    """Halo exchange of this rank's slab with its neighbours (rank - 1 below,
    rank + 1 above, cyclically) over torch.distributed."""
    import torch.distributed as dist
    ws, rank = dist.get_world_size(group), dist.get_rank(group)
    if ws == 1:
        exchange_z_halos_local([t], ng, stream)
        return
    fill_ghosts_xy(t, ng, stream)
    low, high = pack_z(t, ng, 0, stream), pack_z(t, ng, 1, stream)
    from_below, from_above = torch.empty_like(high), torch.empty_like(low)
    up, down = (rank + 1) % ws, (rank - 1) % ws
    # Upward traffic (my top planes become my upper neighbour's lower ghosts) is
    # posted before downward traffic on every rank, and tagged: with two ranks the
    # neighbour above and below is the same peer, and backends that match
    # messages between a pair in posting order (NCCL) or by tag (gloo) then pair
    # each send with the right receive.
    ops = [dist.P2POp(dist.isend, high, up, group, tag=1), dist.P2POp(dist.irecv, from_below, down, group, tag=1),
           dist.P2POp(dist.isend, low, down, group, tag=2), dist.P2POp(dist.irecv, from_above, up, group, tag=2)]
    for r in dist.batch_isend_irecv(ops):
        r.wait()
    unpack_z(t, ng, 0, from_below, stream)
    unpack_z(t, ng, 1, from_above, stream)


def reduce_diagnostics(r: L.DiagResult, group=None) -> tuple:
    """All-reduce of a slab's raw diagnostics: (14 energy sums, n_p_plain,
    n_p_weighted, vel_sum, vel_count) summed over the ranks, and this rank's
    offset in the whole box's pierced list (exclusive prefix sum of n_listed).
    Cell numbers in a slab's list are slab-local: entry + 4 z0 nx ny moves
    them to the box."""
    import torch.distributed as dist
    dev = torch.device("cuda") if dist.get_backend(group) == "nccl" else torch.device("cpu")
    f = torch.tensor(list(r.energy_sums) + [r.vel_sum], dtype=torch.float64, device=dev)
    i = torch.tensor([r.n_p_plain, r.n_p_weighted, r.vel_count, r.n_listed], dtype=torch.int64, device=dev)
    counts = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(dist.get_world_size(group))]
    dist.all_gather(counts, i[3:4].clone(), group=group)
    dist.all_reduce(f, group=group)
    dist.all_reduce(i, group=group)
    rank = dist.get_rank(group)
    offset = int(sum(int(c.item()) for c in counts[:rank]))
    return f[:14].tolist(), int(i[0]), int(i[1]), float(f[14]), int(i[2]), offset
