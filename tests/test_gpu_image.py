"""GPU parity of the image stages around the tile path against the oracle: the Hann overlap blend
(image_pipeline.rs:593-649), the scanner OTF (image_pipeline.rs:825-855) and the Triangle
downsample of supersampled renders (image_pipeline.rs:315-330)."""
import numpy as np
import pytest

from fgrain_gb300 import image as im
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_scanner_otf_is_bit_exact(engine):
    f = np.random.default_rng(3).random((203, 301)).astype(np.float32) * 3.0
    np.testing.assert_array_equal(im.scanner_otf(f), orc.scanner_otf(f))
    taps = (0.1, 0.8, 0.1)
    np.testing.assert_array_equal(im.scanner_otf(f, taps), orc.scanner_otf(f, taps))
    one = np.random.default_rng(4).random((1, 17)).astype(np.float32)  # a single row: clamps in y
    np.testing.assert_array_equal(im.scanner_otf(one), orc.scanner_otf(one))


@pytest.mark.parametrize("ss", [2, 3, 4])
def test_triangle_downsample_is_bit_exact(engine, ss):
    ow, oh = 157, 113
    f = np.random.default_rng(ss).random((oh * ss, ow * ss)).astype(np.float32)
    np.testing.assert_array_equal(im.resize_triangle(f, ow, oh), orc.resize_triangle(f, ow, oh))


def test_upsample_and_odd_ratios(engine):
    f = np.random.default_rng(9).random((50, 70)).astype(np.float32)
    for ow, oh in ((101, 77), (33, 21), (70, 50)):
        np.testing.assert_array_equal(im.resize_triangle(f, ow, oh), orc.resize_triangle(f, ow, oh))


@pytest.mark.parametrize("size,grain", [((700, 500), 2.4), ((1000, 300), 1.1)])
def test_hann_blend_matches_the_oracle(engine, size, grain):
    W, H = size
    grid, step, pad = im.tile_grid(W, H, grain)
    rng = np.random.default_rng(W)
    ds = [rng.random((t.th, t.tw)).astype(np.float32) + 0.05 for t in grid]
    dev = im.blend_tiles(W, H, grid, step, pad, ds)
    ref = orc.blend_tiles(W, H, grid, step, pad, ds)
    # The Hann cosine is correctly rounded on the device and the C library's cosf in the oracle:
    # at most an ulp of the weight apart.
    np.testing.assert_allclose(dev, ref, rtol=2e-7, atol=0)
    # Partition of unity: constant tiles blend to the constant.
    c = [np.full((t.th, t.tw), 0.7, np.float32) for t in grid]
    np.testing.assert_allclose(im.blend_tiles(W, H, grid, step, pad, c), 0.7, rtol=1e-6)
