"""Refinement tagging through the C ABI: the device tagger reproduces the
reference's own StringTagger (golden tags from the reference-built checker)
for the plaquette, Laplacian and radial-gradient criteria in both precisions,
and the n_error_buf buffer, counts and block flags match the oracle."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["f64", "f32"])
@pytest.mark.parametrize("box", ["rand", "ic"])
def test_tagger_matches_reference(axs, golden, prec, box):
    g = golden("tagging.npz")
    v = g[f"{prec}_{box}_state"]
    _, nz, ny, nx = v.shape
    dtype = torch.float64 if prec == "f64" else torch.float32
    lv = axs.PeriodicLevel((nx, ny, nz), 0.5, dtype=dtype)
    lv.set_state(torch.from_numpy(np.ascontiguousarray(v)).cuda())
    for t, (gt, rt) in enumerate(g["thresholds"]):
        tags, n, _ = lv.tag_cells(gt, rt)
        ref = g[f"{prec}_{box}_tags"][t].astype(np.uint8)
        np.testing.assert_array_equal(tags.cpu().numpy(), ref)
        assert n == int(ref.sum())


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_buffer_counts_and_blocks_match_oracle(axs, orc, dtype):
    from axion_strings_adaptive_gb300 import ic
    n, nbuf, block = 32, 2, 8
    s = ic.fourier_state(n, 2.0, seed=8).to(dtype)  # ~1 % pierced cells, ~30 % after the buffer
    lv = axs.PeriodicLevel(n, 0.5, dtype=dtype)
    lv.set_state(s)
    tags, count, flags = lv.tag_cells(n_error_buf=nbuf, block=block)
    fab = orc.to_fab(s.cpu().numpy(), 2)
    ref = orc.tag_cells(fab, 2, 0.5, n_error_buf=nbuf)
    np.testing.assert_array_equal(tags.cpu().numpy(), ref)
    assert count == int(ref.sum()) and 0 < count < n ** 3
    nb = n // block
    ref_flags = ref.reshape(nb, block, nb, block, nb, block).max(axis=(1, 3, 5))
    np.testing.assert_array_equal(flags.cpu().numpy(), ref_flags)


def _block_flags(tags, block):
    nz, ny, nx = tags.shape
    nbz, nby, nbx = (-(-nz // block), -(-ny // block), -(-nx // block))
    out = np.zeros((nbz, nby, nbx), dtype=np.uint8)
    for k in range(nbz):
        for j in range(nby):
            for i in range(nbx):
                out[k, j, i] = tags[k * block:(k + 1) * block, j * block:(j + 1) * block,
                                    i * block:(i + 1) * block].max()
    return out


@pytest.mark.parametrize("shape,nbuf,block", [
    ((64, 24, 20), 5, 16),   # bit-packed buffer: two words per row
    ((64, 24, 20), 33, 12),  # a buffer wider than a word; blocks that straddle words
    ((32, 16, 12), 40, 8),   # one word per row, the buffer wraps the row more than once
    ((64, 24, 20), 0, 16),   # no buffer: count and flags from the packed tags
    ((96, 8, 8), 1, 48),     # blocks wider than a word
    ((36, 20, 16), 3, 6),    # rows of part words: the byte-array passes
])
def test_buffer_shapes_and_block_sizes_match_oracle(axs, orc, shape, nbuf, block):
    from axion_strings_adaptive_gb300 import ic
    nx, ny, nz = shape
    s = ic.fourier_state(shape, 2.5, seed=17)
    lv = axs.PeriodicLevel(shape, 0.5, dtype=torch.float64)
    lv.set_state(s)
    tags, count, flags = lv.tag_cells(n_error_buf=nbuf, block=block)
    ref = orc.tag_cells(orc.to_fab(s.cpu().numpy(), 2), 2, 0.5, n_error_buf=nbuf)
    np.testing.assert_array_equal(tags.cpu().numpy(), ref)
    assert count == int(ref.sum()) and 0 < count
    np.testing.assert_array_equal(flags.cpu().numpy().reshape(-1), _block_flags(ref, block).reshape(-1))
