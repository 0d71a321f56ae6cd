"""The z-slab protocol on CPU ranks (world_size 2, gloo): each rank holds one z
slab of a periodic box as an AMReX-layout FAB, exchanges its halo planes with
its neighbour over torch.distributed, evaluates the counts, energy sums and
velocity sums of its slab with the CPU oracle (ghost-cell boundary), and the
ranks combine them with slabs.reduce_diagnostics (the all-reduce of the 18 raw
scalars and the pierced-list prefix sum). Rank 0 checks the result against the
oracle on the whole box. The oracle is the compute here; the GPU entry points
of the same seam are tested in tests/test_gpu_slabs.py."""
import os
import sys

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHAPE, CUTS, NG, SEED = (20, 16, 14), (0, 6, 14), 2, 41


def _state():
    rng = np.random.default_rng(SEED)
    nx, ny, nz = SHAPE
    return rng.standard_normal((4, nz, ny, nx)) * np.array([1.0, 1.0, 0.3, 0.3])[:, None, None, None]


def _worker(rank, ws, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    from axion_strings_adaptive_gb300 import _lib as L
    from axion_strings_adaptive_gb300.slabs import reduce_diagnostics
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        O.lib()
        v = _state()
        z0, z1 = CUTS[rank], CUTS[rank + 1]
        nz = z1 - z0
        fab = np.zeros(O.fab_shape(SHAPE[0], SHAPE[1], nz, NG), dtype=np.float64)
        fab[:, NG:NG + nz, NG:-NG, NG:-NG] = v[:, z0:z1]
        # x/y ghosts of the valid planes, periodic within the slab
        fab[:, NG:NG + nz, :, :NG] = fab[:, NG:NG + nz, :, -2 * NG:-NG]
        fab[:, NG:NG + nz, :, -NG:] = fab[:, NG:NG + nz, :, NG:2 * NG]
        fab[:, NG:NG + nz, :NG, :] = fab[:, NG:NG + nz, -2 * NG:-NG, :]
        fab[:, NG:NG + nz, -NG:, :] = fab[:, NG:NG + nz, NG:2 * NG, :]
        # halo planes: my top planes go up, my bottom planes go down (same posting
        # order and tags as slabs.exchange_z_halos)
        low = torch.from_numpy(np.ascontiguousarray(fab[:, NG:2 * NG]))
        high = torch.from_numpy(np.ascontiguousarray(fab[:, nz:nz + NG]))
        below, above = torch.empty_like(high), torch.empty_like(low)
        up, down = (rank + 1) % ws, (rank - 1) % ws
        ops = [dist.P2POp(dist.isend, high, up, tag=1), dist.P2POp(dist.irecv, below, down, tag=1),
               dist.P2POp(dist.isend, low, down, tag=2), dist.P2POp(dist.irecv, above, up, tag=2)]
        for r in dist.batch_isend_irecv(ops):
            r.wait()
        fab[:, :NG] = below.numpy()
        fab[:, nz + NG:] = above.numpy()
        R, lam, RpR, m_r = 1.1, 1.3, 0.4, 1.14
        plain, weighted, w = O.count_plaquettes(fab, NG, want_windings=True)
        sums = O.energy_sums(fab, NG, 0.5, R, lam, RpR, O.MASK_A, 0.8)
        vs, vc = O.velocity(fab, NG, R, RpR, m_r)
        res = L.DiagResult()
        for q in range(14):
            res.energy_sums[q] = sums[q]
        res.vel_sum, res.vel_count, res.n_p_plain, res.n_p_weighted = vs, vc, plain, weighted
        cells = np.arange(w.shape[0] * w.shape[1] * w.shape[2]).reshape(w.shape[:3])
        local = np.sort(np.concatenate([4 * cells[w[..., pl] != 0] + pl for pl in range(3)]))
        res.n_listed = len(local)
        esum, p_, w_, vsum, vcnt, offset = reduce_diagnostics(res)
        out.put((rank, esum, p_, w_, vsum, vcnt, offset, (local + 4 * z0 * SHAPE[0] * SHAPE[1]).tolist()))
    finally:
        dist.destroy_process_group()


def test_slab_reduction_over_gloo_matches_the_whole_box():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted([q.get(timeout=120) for _ in range(2)], key=lambda g: g[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    O.lib()
    fab = O.to_fab(_state(), NG)
    plain, weighted, w = O.count_plaquettes(fab, NG, want_windings=True)
    sums = O.energy_sums(fab, NG, 0.5, 1.1, 1.3, 0.4, O.MASK_A, 0.8)
    vs, vc = O.velocity(fab, NG, 1.1, 0.4, 1.14)
    cells = np.arange(w.shape[0] * w.shape[1] * w.shape[2]).reshape(w.shape[:3])
    whole_list = np.sort(np.concatenate([4 * cells[w[..., pl] != 0] + pl for pl in range(3)]))
    for rank, esum, p_, w_, vsum, vcnt, offset, entries in got:
        assert (p_, w_, vcnt) == (plain, weighted, vc)
        np.testing.assert_allclose(esum, sums[:14], rtol=1e-12)
        assert abs(vsum - vs) <= 1e-12 * abs(vs)
    assert got[0][6] == 0 and got[1][6] == len(got[0][7])  # prefix-sum offsets
    np.testing.assert_array_equal(np.sort(np.array(got[0][7] + got[1][7])), whole_list)
