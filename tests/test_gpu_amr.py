"""Refined patches through the C ABI (the scale path's fine level):
* a patch step with its ghost ring filled from a uniform fine level equals that
  level's own step on the same cells, bit for bit;
* the ring interpolation is exact for fields that are quartic polynomials
  around the patch, and equals a numpy restatement on a random field;
* with every block refined the patches evolve exactly as a uniform level of
  twice the resolution (the coarse level never reaches their rings);
* the homogeneous solution psi = R(tau), Pi = R'(tau) survives subcycling;
* composite diagnostics count a straight string pair on the fine level;
* a mid-step ring fill copies neighbour-owned cells and blends the coarse
  states in time as a numpy restatement does;
* the batched pass over all patches equals per-patch diagnostics passes."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _ring_from_level(patches, q, origin, fine):
    """Fill patch q (valid + ring) from a periodic fine field (4, N, N, N)."""
    n = patches.n
    lay = patches.layout
    N = fine.shape[-1]
    box = patches.box(q)
    ox, oy, oz = origin
    xs = (ox + np.arange(-6, n + 6)) % N
    ys = (oy + np.arange(-4, n + 4)) % N
    zs = (oz + np.arange(-4, n + 4)) % N
    sub = fine[:, zs][:, :, ys][:, :, :, xs]
    box[:, lay.z_offset - 4:lay.z_offset + n + 4, lay.y_offset - 4:lay.y_offset + n + 4,
        lay.x_offset - 6:lay.x_offset + n + 6] = sub


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("n", [32, 64])
def test_patch_step_matches_uniform_level(axs, dtype, n):
    """Patch side 32 takes the fused step (one thread-block cluster of tiles per
    patch) in both precisions, side 64 the fused step in FP32 (8 tiles) and the
    two separate sweeps in FP64; all equal the uniform level."""
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.amr import Patches
    Nf, dx = 2 * n, 0.25
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    s0 = ic.fourier_state(Nf, 6.0 * Nf / 64, seed=3)
    s0[2:] = 0.1 * torch.randn_like(s0[2:])
    s0 = s0.to(dtype)
    fine = axs.PeriodicLevel(Nf, dx, dtype=dtype)
    fine.set_state(s0)
    origins = [(0, 0, 0), (n, 0, n), (n, n, 0)]
    p = Patches(n, len(origins), dx, dtype=dtype)
    for q, o in enumerate(origins):
        _ring_from_level(p, q, o, s0.cuda())
    p.step(bg, 1.0, 0.3, 0.05)
    p.device_status()
    fine.advance(bg, 1.0, 0.3, 0.05, 1)
    ref = fine.get_state()
    for q, (ox, oy, oz) in enumerate(origins):
        assert torch.equal(p.valid(q), ref[:, oz:oz + n, oy:oy + n, ox:ox + n]), q


def _quartic_weights():
    w = np.zeros((2, 5))
    for s, xi in enumerate((-0.25, 0.25)):
        for k in range(5):
            num = den = 1.0
            for m in range(5):
                if m != k:
                    num *= xi - (m - 2)
                    den *= k - m
            w[s, k] = num / den
    return w


def test_interpolation_quartic_exact_and_restated(axs):
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 64, 16
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float64)
    c = (np.arange(N) + 0.5)
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    xc = 24.0
    poly = lambda x, y, z: (1.0 + 0.3 * (x - xc) - 0.02 * (x - xc) ** 4) * (0.5 + 0.1 * (y - xc) ** 3) + \
        0.01 * (z - xc) ** 4 - 0.2 * (z - xc) * (y - xc)
    st = np.stack([poly(X, Y, Z), poly(Y, Z, X), poly(Z, X, Y), 0.5 * poly(X, Z, Y)])
    coarse.set_state(torch.from_numpy(st).cuda())
    two = TwoLevel(coarse, block)
    two.set_blocks(np.array([[1, 1, 1]]))  # coarse cells 16..31: its 5-point stencils stay inside 11..36
    p = two.patches
    box = p.box(0).cpu().numpy()
    n, lay = p.n, p.layout
    f = (np.arange(-4, n + 4) + 0.5) * 0.5 + 16.0  # fine centres in coarse units (coarse x = c + 0.5)
    fx = (np.arange(-6, n + 6) + 0.5) * 0.5 + 16.0
    FZ, FY, FX = np.meshgrid(f, f, fx, indexing="ij")
    exact = np.stack([poly(FX, FY, FZ), poly(FY, FZ, FX), poly(FZ, FX, FY), 0.5 * poly(FX, FZ, FY)])
    got = box[:, lay.z_offset - 4:lay.z_offset + n + 4, lay.y_offset - 4:lay.y_offset + n + 4,
              lay.x_offset - 6:lay.x_offset + n + 6]
    np.testing.assert_allclose(got, exact, rtol=1e-12, atol=1e-10 * np.abs(exact).max())

    # a random field: the device interpolation equals a numpy restatement
    rng = np.random.default_rng(5)
    st = rng.standard_normal((4, N, N, N))
    coarse.set_state(torch.from_numpy(st).cuda())
    two.set_blocks(np.zeros((0, 3)))
    two.set_blocks(np.array([[3, 0, 2]]))  # wraps in x and y around the periodic seam
    w = _quartic_weights()
    box = two.patches.box(0).cpu().numpy()
    for (x, y, z) in [(0, 0, 0), (-6, 5, -4), (n + 5, n + 3, 7), (13, -1, n + 2)]:
        gx, gy, gz = 3 * 32 + x, 0 * 32 + y, 2 * 32 + z
        val = 0.0
        for k in range(5):
            for j in range(5):
                for i in range(5):
                    cx, cy, cz = (gx // 2 + i - 2) % N, (gy // 2 + j - 2) % N, (gz // 2 + k - 2) % N
                    val += w[gx % 2, i] * w[gy % 2, j] * w[gz % 2, k] * st[0, cz, cy, cx]
        got = box[0, z + lay.z_offset, y + lay.y_offset, x + lay.x_offset]
        assert got == pytest.approx(val, rel=1e-12, abs=1e-12)


def test_fully_refined_patches_evolve_as_uniform_fine_level(axs):
    from axion_strings_adaptive_gb300 import ic
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 32, 16
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float32)
    coarse.set_state(ic.fourier_state(N, 5.0, seed=9).float())
    two = TwoLevel(coarse, block)
    nb = N // block
    two.set_blocks(np.array([[x, y, z] for z in range(nb) for y in range(nb) for x in range(nb)]))
    n = two.patches.n
    fine = axs.PeriodicLevel(2 * N, 0.25, dtype=torch.float32)
    full = torch.empty((4, 2 * N, 2 * N, 2 * N), dtype=torch.float32, device="cuda")
    for q, (bx, by, bz) in enumerate(two.blocks):
        full[:, bz * n:(bz + 1) * n, by * n:(by + 1) * n, bx * n:(bx + 1) * n] = two.patches.valid(q)
    fine.set_state(full)
    two.advance(bg, 1.0, 0.0, 0.1, 3)
    two.device_status()
    fine.advance(bg, 1.0, 0.0, 0.05, 6)
    ref = fine.get_state()
    for q, (bx, by, bz) in enumerate(two.blocks):
        assert torch.equal(two.patches.valid(q), ref[:, bz * n:(bz + 1) * n, by * n:(by + 1) * n,
                                                    bx * n:(bx + 1) * n]), q


def test_homogeneous_solution_survives_subcycling(axs):
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 64, 16
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)  # RD: R = tau, R' = 1, kappa = 0
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float64)
    st = torch.zeros((4, N, N, N), dtype=torch.float64)
    st[0], st[2] = 1.0, 1.0
    coarse.set_state(st.cuda())
    two = TwoLevel(coarse, block)
    two.set_blocks(np.array([[0, 0, 0], [1, 0, 0], [3, 2, 1]]))
    two.advance(bg, 1.0, 0.0, 0.1, 5)
    two.device_status()
    for q in range(two.patches.npatches):
        v = two.patches.valid(q)
        assert torch.allclose(v[0], torch.full_like(v[0], 1.5), rtol=1e-13, atol=0)
        assert torch.allclose(v[2], torch.full_like(v[2], 1.0), rtol=1e-13, atol=0)
        assert float(v[1].abs().max()) < 1e-14 and float(v[3].abs().max()) < 1e-14


def test_composite_diagnostics_straight_strings(axs):
    from test_gpu_physics import straight_string_pair
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, nz, dx, block = 64, 64, 0.5, 16
    bg = axs.Background.expanding(2.0, 1.0)
    v = bg.values(1.0)
    coarse = axs.PeriodicLevel((N, N, nz), dx, dtype=torch.float64)
    coarse.set_state(torch.from_numpy(straight_string_pair(N, nz, dx, v.R, v.m_r, v.R_prime_over_R)).cuda())
    two = TwoLevel(coarse, block)
    nref = two.regrid(n_error_buf=4)
    assert 0 < nref < (N // block) ** 2 * (nz // block)
    d = two.diagnostics(bg, 1.0)
    # both strings run through refined blocks only: 2 pierced fine xy plaquettes per fine layer
    assert d.n_p_plain == 2 * (2 * nz) and d.n_patches == nref
    d0 = coarse.diagnostics(bg, 1.0)
    # the same string length: twice the plaquettes at half the spacing (ell = (2/3) N_p dx)
    assert d.xi_plain == pytest.approx(d0.xi_plain, rel=1e-12)
    # the string finder alone (masked coarse level and the patches) counts the same
    ds = two.diagnostics(bg, 1.0, strings_only=True)
    assert (ds.n_p_plain, ds.n_p_weighted) == (d.n_p_plain, d.n_p_weighted)


def test_time_interpolated_ring_and_neighbour_copies(axs):
    """Mid-step ring fill (theta > 0): cells a neighbouring patch owns are copied
    from it; the others equal a numpy restatement of the cubic-Hermite (psi,
    with Pi as its derivative) / linear (Pi) blend of the quartic spatial
    interpolation of the coarse states at both ends of the coarse step."""
    import ctypes as C
    from axion_strings_adaptive_gb300 import _lib as L
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block, theta, cdt = 64, 16, 0.37, 0.1
    rng = np.random.default_rng(11)
    old = rng.standard_normal((4, N, N, N))
    new = old + 0.1 * rng.standard_normal((4, N, N, N))
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float64)
    coarse.set_state(torch.from_numpy(new).cuda())
    two = TwoLevel(coarse, block)
    start = axs.PeriodicLevel(N, 0.5, dtype=torch.float64)
    start.set_state(torch.from_numpy(old).cuda())
    two.old_state.copy_(start.state)
    blocks = np.array([[3, 0, 2], [0, 0, 2], [3, 3, 2]])  # x-neighbours across the seam, a y-neighbour across it
    two.set_blocks(blocks)
    p = two.patches
    p.state[:, :] = 0
    for q in range(p.npatches):
        p.valid(q).copy_(torch.from_numpy(rng.standard_normal((4, p.n, p.n, p.n))).cuda())
    L.call("axs_patches_fill", C.byref(p.c), C.byref(two._map()), C.byref(two.old_c), C.byref(coarse.c), theta, cdt,
           0, None)
    torch.cuda.synchronize()
    w = _quartic_weights()
    n, lay = p.n, p.layout
    boxes = [p.box(q).cpu().numpy() for q in range(p.npatches)]
    s, s2, s3 = theta, theta ** 2, theta ** 3
    h00, h10, h01, h11 = 2 * s3 - 3 * s2 + 1, (s3 - 2 * s2 + s) * cdt, -2 * s3 + 3 * s2, (s3 - s2) * cdt
    nf = 2 * N

    def interp(field, gx, gy, gz):
        val = 0.0
        for k in range(5):
            for j in range(5):
                for i in range(5):
                    cx, cy, cz = (gx // 2 + i - 2) % N, (gy // 2 + j - 2) % N, (gz // 2 + k - 2) % N
                    val += w[gx % 2, i] * w[gy % 2, j] * w[gz % 2, k] * field[cz, cy, cx]
        return val

    q = 0  # block (3, 0, 2): its +x ring is patch 1's valid cells, its -y ring patch 2's
    # two cells owned by neighbours ((n+2, 5, 7) and (4, -3, 9)), four interpolated
    cells = [(n + 2, 5, 7), (n + 5, n + 3, -4), (-6, 0, 0), (4, -3, 9), (13, -1, n + 2), (n - 1, n + 3, -2)]
    for (x, y, z) in cells:
        gx, gy, gz = (3 * n + x) % nf, (0 * n + y) % nf, (2 * n + z) % nf
        got = boxes[q][:, z + lay.z_offset, y + lay.y_offset, x + lay.x_offset]
        owner = {(0, 0, 2): 1, (3, 3, 2): 2}.get((gx // n, gy // n, gz // n))
        if owner is not None:
            lx, ly, lz = gx % n, gy % n, gz % n
            want = boxes[owner][:, lz + lay.z_offset, ly + lay.y_offset, lx + lay.x_offset]
            assert np.array_equal(got, want), (x, y, z)
            continue
        for c in range(2):
            p0, p1 = interp(old[c], gx, gy, gz), interp(new[c], gx, gy, gz)
            q0, q1 = interp(old[2 + c], gx, gy, gz), interp(new[2 + c], gx, gy, gz)
            assert got[c] == pytest.approx(h00 * p0 + h10 * q0 + h01 * p1 + h11 * q1, rel=1e-12, abs=1e-12)
            assert got[2 + c] == pytest.approx((1 - s) * q0 + s * q1, rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batched_patch_diagnostics_match_per_patch_passes(axs, dtype):
    """axs_patches_diagnostics (one pass over all patches) equals the sum of
    per-patch axs_diagnostics passes: counts, velocity count and the pierced set
    exactly, sums to rounding."""
    import ctypes as C
    from axion_strings_adaptive_gb300 import _lib as L, ic
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 64, 16
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)
    coarse = axs.PeriodicLevel(N, 0.5, dtype=dtype)
    coarse.set_state(ic.fourier_state(N, 8.0, seed=21).to(dtype))
    two = TwoLevel(coarse, block)
    two.set_blocks(np.array([[0, 0, 0], [1, 0, 0], [3, 2, 1], [2, 2, 3], [0, 3, 3]]))
    two.advance(bg, 1.0, 0.0, 0.1, 2)
    L.call("axs_patches_fill", C.byref(two.patches.c), C.byref(two._map()), C.byref(coarse.c), None, 0.0, 0.0, 0,
           None)
    p = two.patches
    v = bg.values(1.2)
    prm = L.DiagParams(p.dx, v.R, v.lambda_, v.R_prime_over_R, v.m_r, L.MASK_A, 0.8, L.BOUNDARY_GHOSTS, 1, 1, 1, 0)
    cap = 1 << 16
    got, lst = p.diagnostics(prm, list_capacity=cap)
    nbytes = C.c_int64()
    L.call("axs_diagnostics_scratch_bytes", p.n, p.n, p.n, C.byref(nbytes))
    scratch = torch.zeros(nbytes.value, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    sums, cnts, vsum, pierced = np.zeros(14), np.zeros(4, dtype=np.int64), 0.0, set()
    ncell = p.n ** 3
    for q in range(p.npatches):
        res = torch.zeros(C.sizeof(L.DiagResult), dtype=torch.uint8, device="cuda")
        one = torch.zeros(cap, dtype=torch.int64, device="cuda")
        L.call("axs_diagnostics", C.byref(p.fab(q)), C.byref(prm), None, res.data_ptr(), one.data_ptr(), cap,
               scratch.data_ptr(), scratch.numel(), s)
        r = L.DiagResult.from_buffer_copy(res.cpu().numpy().tobytes())
        sums += np.array(list(r.energy_sums))
        cnts += [r.n_p_plain, r.n_p_weighted, r.vel_count, r.n_near_tie]
        vsum += r.vel_sum
        e = one[:r.n_listed].cpu().numpy()
        pierced |= set((4 * (q * ncell + e // 4) + e % 4).tolist())
    assert cnts[0] > 0
    assert [got.n_p_plain, got.n_p_weighted, got.vel_count, got.n_near_tie] == cnts.tolist()
    assert set(lst.cpu().numpy().tolist()) == pierced and got.n_listed == len(pierced)
    np.testing.assert_allclose(np.array(list(got.energy_sums)), sums, rtol=1e-12)
    assert got.vel_sum == pytest.approx(vsum, rel=1e-12)
    if dtype == torch.float32:
        # FP32 per-cell terms over all patches (the energy kernel and the velocity finder
        # on ghost-ring boxes): exact counts and pierced set, sums to FP32 accuracy
        prm32 = L.DiagParams(p.dx, v.R, v.lambda_, v.R_prime_over_R, v.m_r, L.MASK_A, 0.8, L.BOUNDARY_GHOSTS,
                             1, 1, 1, 1)
        g32, l32 = p.diagnostics(prm32, list_capacity=cap)
        assert [g32.n_p_plain, g32.n_p_weighted, g32.vel_count, g32.n_near_tie] == cnts.tolist()
        assert set(l32.cpu().numpy().tolist()) == pierced
        np.testing.assert_allclose(np.array(list(g32.energy_sums)), sums, rtol=2e-6)
        assert g32.energy_sums[13] == sums[13]
        assert g32.vel_sum == pytest.approx(vsum, rel=1e-5)
    # the string finder alone over all patches: the same counts and pierced set
    prm_s = L.DiagParams(p.dx, v.R, v.lambda_, v.R_prime_over_R, v.m_r, L.MASK_A, 0.8, L.BOUNDARY_GHOSTS, 0, 1, 0, 0)
    alone, lst_s = p.diagnostics(prm_s, list_capacity=cap)
    assert [alone.n_p_plain, alone.n_p_weighted, alone.n_near_tie] == [got.n_p_plain, got.n_p_weighted,
                                                                        got.n_near_tie]
    assert set(lst_s.cpu().numpy().tolist()) == pierced and alone.n_listed == len(pierced)


def test_regrid_keeps_the_fine_data_of_blocks_that_stay_refined(axs):
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 64, 16
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float32)
    coarse.set_state(torch.randn((4, N, N, N)).cuda())
    two = TwoLevel(coarse, block)
    two.set_blocks(np.array([[0, 0, 0], [1, 2, 3], [3, 3, 1]]))
    marks = {}
    for q, b in enumerate(two.blocks):
        two.patches.valid(q).fill_(float(q + 7))
        marks[tuple(b)] = float(q + 7)
    two.set_blocks(np.array([[2, 0, 0], [3, 3, 1], [0, 0, 0], [1, 1, 1]]))  # two kept, two new, one dropped
    for q, b in enumerate(two.blocks):
        v = two.patches.valid(q)
        if tuple(b) in marks:
            assert bool((v == marks[tuple(b)]).all()), tuple(b)
        else:  # interpolated from the coarse level
            assert not bool((v == 7.0).any()) and float(v.abs().max()) > 0.0


def test_regrid_in_place_moves_kept_patches_into_free_slots(axs):
    """Six patches (arena laid out for 8 slots), then a set that drops the four
    lowest slots, keeps the two highest and adds one: the regrid stays in the
    arena, moves the kept patches down into slots 0 and 1 with their data, and
    the new patch interpolates the coarse level; then a set past the capacity
    moves everything to a new arena, data intact."""
    from axion_strings_adaptive_gb300.amr import TwoLevel
    N, block = 64, 16
    coarse = axs.PeriodicLevel(N, 0.5, dtype=torch.float32)
    coarse.set_state(torch.randn((4, N, N, N)).cuda())
    two = TwoLevel(coarse, block, headroom=1.34)
    first = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0], [0, 1, 0], [1, 1, 0]])
    two.set_blocks(first)
    assert two.patches.capacity == 9
    arena = two.patches.storage.data_ptr()
    for q in range(6):
        two.patches.valid(q).fill_(float(q + 7))
    marks = {tuple(b): float(q + 7) for q, b in enumerate(two.blocks)}
    two.set_blocks(np.array([[1, 1, 0], [3, 3, 3], [0, 1, 0]]))
    assert two.patches.storage.data_ptr() == arena and two.patches.npatches == 3
    for q, b in enumerate(two.blocks):
        v = two.patches.valid(q)
        if tuple(b) in marks:
            assert bool((v == marks[tuple(b)]).all()), tuple(b)
        else:
            assert not bool((v >= 7.0).all()) and float(v.abs().max()) > 0.0
    assert int((two._block_patch >= 0).sum()) == 3
    for q, b in enumerate(two.blocks):
        assert int(two._block_patch[b[2], b[1], b[0]]) == q
    kept = {tuple(b): two.patches.valid(q).clone() for q, b in enumerate(two.blocks)}
    bigger = np.array([[i % 4, (i // 4) % 4, i // 16] for i in range(12)] + [[3, 3, 3]])
    bigger = np.unique(np.concatenate([bigger, np.array([[1, 1, 0], [0, 1, 0]])]), axis=0)
    two.set_blocks(bigger)
    assert two.patches.npatches == len(bigger) and two.patches.capacity >= len(bigger)
    for q, b in enumerate(two.blocks):
        if tuple(b) in kept:
            assert torch.equal(two.patches.valid(q), kept[tuple(b)]), tuple(b)


def test_patch_counts_past_the_grid_and_two_sweep_limits(axs):
    """70 000 patches: past the two-sweep step's 32 767 (its work items carry box
    numbers in 16 bits) and past one grid's 65 535 z slices (the fused step then
    launches in chunks). A homogeneous radiation-era solution (psi = R = tau,
    Pi = R' = 1) survives a subcycled coarse step in every patch, the last ones
    included."""
    from axion_strings_adaptive_gb300.amr import TwoLevel
    nx, ny, nz, block = 1024, 1024, 512, 16
    bg = axs.Background.expanding(2.0, 1.0, lambda0=2.0)  # RD: R = tau, R' = 1, kappa = 0
    coarse = axs.PeriodicLevel((nx, ny, nz), 0.5, dtype=torch.float32, pierced_capacity=1)
    st = torch.zeros((4, nz, ny, nx), dtype=torch.float32, device="cuda")
    st[0], st[2] = 1.0, 1.0
    coarse.set_state(st)
    del st
    two = TwoLevel(coarse, block, headroom=1.0)
    nbx, nby = nx // block, ny // block
    q = np.arange(70000)
    two.set_blocks(np.stack([q % nbx, (q // nbx) % nby, q // (nbx * nby)], axis=1))
    assert two.patches.npatches == 70000 and two.patches.layout.work_bytes == 0
    two.advance(bg, 1.0, 0.0, 0.1, 1)
    two.device_status()
    p, n = two.patches, two.patches.n
    lay = p.layout
    boxes = p.state.view(4, p.npatches, n + 8, n + 8, lay.jstride)
    valid = boxes[:, :, lay.z_offset:lay.z_offset + n, lay.y_offset:lay.y_offset + n,
                  lay.x_offset:lay.x_offset + n]
    assert float((valid[0] - 1.1).abs().max()) < 2e-6
    assert float((valid[2] - 1.0).abs().max()) < 2e-6
    assert float(valid[1].abs().max()) < 1e-6 and float(valid[3].abs().max()) < 1e-6
