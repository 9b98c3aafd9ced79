"""GPU tests of the fast-approximation mode (the reference's wgpu tile model on the device)
against the oracle's restatement: d_neg and every grid cell bit for bit, one tile or many."""
import numpy as np
import pytest

from fgrain_gb300 import fast
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def blurred(h, w, seed, scale=1.0):
    from scipy.ndimage import gaussian_filter

    a = np.random.default_rng(seed).random((h, w))
    return (np.clip(gaussian_filter(a, 4, mode="reflect") * 3 - 1, 0, 1) * scale).astype(np.float32)


CASES = [("tri-x", 1 / 2.4, 96, 80, 1.0, 0.0), ("t-max", 1 / 1.1, 64, 64, 1.0, 0.5), ("hp5", 1 / 1.8, 72, 90, 1.3, 1.0),
         ("tri-x-1600", 1 / 2.2, 50, 40, 1.0, 2.0), ("tri-x", 1 / 2.4, 40, 40, 20.0, 0.0)]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_tile_bit_exact_with_oracle(engine, case):
    preset, px, tw, th, exposure, push = CASES[case]
    p = fast.tile_params_fast(preset, px, tw, th, exposure, push, 11 + case)
    tile = blurred(th, tw, case)
    d, cells = fast.render_tile_fast(tile, p, engine, cells=True)
    do, co = orc.fast_tile(p, tile)
    for f in ("pos", "dims_exp", "rot", "flags"):
        np.testing.assert_array_equal(cells[f], co[f], err_msg=f)
    np.testing.assert_array_equal(d, do)


def test_large_tile_with_scaled_grid(engine):
    p = fast.tile_params_fast("tri-x", 2.0, 384, 120, 1.0, 0.0, 5)
    (w, h, dd), cs = fast.fast_grid(p)
    assert w == 512 and cs > 1.2
    tile = blurred(120, 384, 9)
    d = fast.render_tile_fast(tile, p, engine)
    do, _ = orc.fast_tile(p, tile)
    np.testing.assert_array_equal(d, do)


def test_batch_equals_single_tiles(engine):
    ps = [fast.tile_params_fast(pr, px, tw, th, ex, pu, 100 + k) for k, (pr, px, tw, th, ex, pu) in enumerate(CASES)]
    tiles = [blurred(p.height_px, p.width_px, 50 + k) for k, p in enumerate(ps)]
    batch = fast.render_tiles_fast(ps, tiles, engine)
    for p, t, b in zip(ps, tiles, batch):
        np.testing.assert_array_equal(b, fast.render_tile_fast(t, p, engine))


def test_dark_tile_is_base_density(engine):
    p = fast.tile_params_fast("hp5", 1 / 1.8, 33, 21, 1.0, 0.0, 1)
    d = fast.render_tile_fast(np.zeros((21, 33), np.float32), p, engine)
    assert (d == np.float32(0.05)).all()


@pytest.mark.parametrize("tw,th", [(1, 1), (1, 9), (13, 2)])
def test_tiny_tiles_bit_exact(engine, tw, th):
    p = fast.tile_params_fast("hp5", 1 / 1.8, tw, th, 1.0, 0.0, 4)
    tile = np.full((th, tw), 0.8, np.float32)
    d, cells = fast.render_tile_fast(tile, p, engine, cells=True)
    do, co = orc.fast_tile(p, tile)
    np.testing.assert_array_equal(d, do)
    np.testing.assert_array_equal(cells["flags"], co["flags"])
