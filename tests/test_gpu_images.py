"""GPU tests of whole images through the batched tile path: the colour driver (three independent
layers with seed offsets, image_pipeline.rs:1017-1085) and a mixed batch of images of different
stocks, sizes, pushes and supersampling factors in one graph launch (the batched configuration)."""
import numpy as np
import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import image as im

pytestmark = pytest.mark.gpu


def blurred(h, w, seed, sigma=8.0):
    from scipy.ndimage import gaussian_filter

    a = np.random.default_rng(seed).random((h, w))
    return (np.clip(gaussian_filter(a, sigma, mode="reflect"), 0, None) ** 2.2).astype(np.float32)


def test_color_layers_are_independent_runs_with_offset_seeds(engine):
    H, W = 400, 700
    rgb = np.stack([blurred(H, W, s) for s in (1, 2, 3)])
    out = im.render_color_image(rgb, "tri-x", 2.4, 0.0, 5, engine)
    assert out.shape == (3, H, W)
    for c, off in enumerate(im.COLOR_SEED_OFFSETS):
        single = im.render_bw_image(rgb[c], "tri-x", 2.4, 0.0, 5 + off, engine)
        np.testing.assert_array_equal(out[c], single)
    assert not np.array_equal(out[0], out[1])
    assert np.isfinite(out).all() and (out >= 0.05 - 1e-6).all()


def test_mixed_images_in_one_batch_equal_their_own_runs(engine):
    """Images of different stocks, sizes, pushes and supersampling factors share one batch (one
    graph launch, autotuned); each image's tiles equal the tiles of its own batch."""
    rng = np.random.default_rng(0)
    stocks = [("tri-x", 2.4), ("t-max", 1.1), ("hp5", 1.8)]
    params, tiles, spans = [], [], []
    for k in range(6):
        side = int(round(np.exp(rng.uniform(np.log(64), np.log(256)))))
        ss = int(rng.integers(1, 3))
        stock, grain = stocks[k % 3]
        push = float(rng.uniform(0, 3))
        exp = blurred(side * ss, side * ss, k, 4.0 * ss)
        grid, _, _ = im.tile_grid(side * ss, side * ss, grain)
        p = im.image_tile_params(stock, grain, grid, 1.0, push, k)
        t = [np.ascontiguousarray(exp[g.y_start:g.y_start + g.th, g.x_start:g.x_start + g.tw]) for g in grid]
        spans.append((len(params), len(p)))
        params += p
        tiles += t
    b = fg.Batch(params, engine, use_graph=True, autotune=True)
    d = im.render_tiles(params, tiles, engine, batch=b)
    b.close()
    for (s, n) in spans:
        own = im.render_tiles(params[s:s + n], tiles[s:s + n], engine)
        for x, y in zip(d[s:s + n], own):
            np.testing.assert_array_equal(x, y)
