"""The z-slab seam on one GPU: a periodic box cut into z slabs held by one
process, with halos exchanged through the library's pack / unpack entry points
(axs_fill_periodic_ghosts_xy, axs_fab_pack_z_planes, axs_fab_unpack_z_planes).
The RHS on the slabs equals the whole box's bit for bit, a drop-in RK4 step
with one exchange per stage equals the whole box's step bit for bit, and the
slabs' diagnostics, summed as an all-reduce would, equal the whole box's
(counts and pierced list exactly, sums to rounding)."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NG = 2


def _split(axs, whole_valid, cuts, dtype):
    slabs = []
    for z0, z1 in zip(cuts[:-1], cuts[1:]):
        t = axs.new_fab((whole_valid.shape[3], whole_valid.shape[2], z1 - z0), NG, dtype=dtype)
        axs.valid(t, NG).copy_(whole_valid[:, z0:z1])
        slabs.append(t)
    return slabs


def _box(axs, shape, dtype, seed):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((4, nz, ny, nx)) * np.array([1.0, 1.0, 0.3, 0.3])[:, None, None, None]
    return torch.from_numpy(v).to(dtype).cuda()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("cuts", [(0, 10, 20), (0, 4, 9, 20)])
def test_slab_rhs_and_rk4_step_equal_the_whole_box(axs, dtype, cuts):
    from axion_strings_adaptive_gb300 import slabs as S
    shape, dx, dt = (32, 24, 20), 0.5, 0.1
    v = _box(axs, shape, dtype, 3)
    bg = axs.Background.expanding(1.5, 1.0, lambda0=2.0)
    whole = axs.new_fab(shape, NG, dtype=dtype)
    axs.valid(whole, NG).copy_(v)
    parts = _split(axs, v, cuts, dtype)

    def rk4_step(fabs, exchange, t):
        uold = [f.clone() for f in fabs]
        us = [torch.zeros_like(f) for f in fabs]
        ks = [[torch.zeros_like(f) for _ in range(4)] for f in fabs]
        for s_, (ts, cs) in enumerate(((t, 0.5 * dt), (t + 0.5 * dt, 0.5 * dt), (t + 0.5 * dt, dt), (t + dt, None))):
            src = uold if s_ == 0 else us
            exchange(src)
            for b in range(len(fabs)):
                axs.eval_rhs(src[b], ks[b][s_], NG, NG, dx, bg.rhs_coeffs(1.0 + ts))
                if cs is not None:
                    axs.lincomb(us[b], uold[b], cs, ks[b][s_], NG)
        for b in range(len(fabs)):
            axs.rk4_combine(fabs[b], uold[b], *ks[b], NG, dt)
        return ks

    k_whole = rk4_step([whole], lambda fs: axs.fill_periodic_ghosts(fs[0], NG), 0.0)
    k_parts = rk4_step(parts, lambda fs: S.exchange_z_halos_local(fs, NG), 0.0)
    for s_ in range(4):  # every stage's RHS, slab by slab
        got = torch.cat([axs.valid(k[s_], NG) for k in k_parts], dim=1)
        assert torch.equal(got, axs.valid(k_whole[0][s_], NG)), s_
    got = torch.cat([axs.valid(f, NG) for f in parts], dim=1)
    assert torch.equal(got, axs.valid(whole, NG))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_slab_diagnostics_reduce_to_the_whole_box(axs, dtype):
    from axion_strings_adaptive_gb300 import slabs as S
    L = axs._lib
    shape, cuts = (24, 20, 18), (0, 7, 18)
    nx, ny, nz = shape
    v = _box(axs, shape, dtype, 9)
    params = L.DiagParams(0.5, 1.1, 1.3, 0.4, 1.14, L.MASK_A, 0.8, L.BOUNDARY_GHOSTS, 1, 1, 1)

    def diag(t):
        f = axs.fab(t, NG)
        ncell = f.nx * f.ny * f.nz
        scratch = torch.zeros(axs.level.scratch_bytes(f.nx, f.ny, f.nz), dtype=torch.uint8, device="cuda")
        res = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device="cuda")
        lst = torch.full((3 * ncell,), -1, dtype=torch.int64, device="cuda")
        L.call("axs_diagnostics", C.byref(f), C.byref(params), None, res.data_ptr(), lst.data_ptr(), lst.numel(),
               scratch.data_ptr(), scratch.numel(), None)
        torch.cuda.synchronize()
        r = L.DiagResult.from_buffer_copy(res.cpu().numpy().tobytes())
        return r, lst[: r.n_listed].cpu().numpy()

    whole = axs.new_fab(shape, NG, dtype=dtype)
    axs.valid(whole, NG).copy_(v)
    axs.fill_periodic_ghosts(whole, NG)
    rw, lw = diag(whole)
    parts = _split(axs, v, cuts, dtype)
    S.exchange_z_halos_local(parts, NG)
    sums, cnt, lists = np.zeros(14), np.zeros(4, dtype=np.int64), []
    vsum = 0.0
    for (z0, z1), t in zip(zip(cuts[:-1], cuts[1:]), parts):
        r, lst = diag(t)
        sums += np.array(r.energy_sums)
        vsum += r.vel_sum
        cnt += np.array([r.n_p_plain, r.n_p_weighted, r.vel_count, r.n_listed])
        lists.append(lst + 4 * z0 * nx * ny)  # slab-local cells into the box's numbering
    assert tuple(cnt) == (rw.n_p_plain, rw.n_p_weighted, rw.vel_count, rw.n_listed)
    np.testing.assert_allclose(sums, list(rw.energy_sums), rtol=1e-12)
    assert vsum == pytest.approx(rw.vel_sum, rel=1e-12)
    np.testing.assert_array_equal(np.sort(np.concatenate(lists)), np.sort(lw))
