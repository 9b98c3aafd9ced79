"""The product's tile grid and tile seeds (fgrain_gb300/image.py) against the oracle's independent
restatement of image_pipeline.rs:377-434 (oracle/oracle.py film_grid, film_tile_seed): every tile's
index, grid position, pixel window and seed, over image sizes, grain sizes, tile sizes and seeds,
including images smaller than one tile and sizes that leave ragged last rows and columns."""
import itertools

import numpy as np
import pytest

from fgrain_gb300 import image as im
from oracle import oracle as orc

SIZES = [(1, 1), (17, 9), (48, 48), (320, 320), (321, 319), (1000, 750), (2048, 2048), (4096, 2731), (16384, 64)]
GRAINS = [0.05, 0.2, 0.5, 0.83, 1.1, 1.8, 2.4, 3.7]
TILE_SIZES = [96, 320, 512]
SEEDS = [0, 42, 2**63 - 1, 2**64 - 1]


@pytest.mark.parametrize("w,h", SIZES)
def test_tile_grid_equals_the_oracle(w, h):
    for grain, ts in itertools.product(GRAINS, TILE_SIZES):
        got, step, pad = im.tile_grid(w, h, grain, ts)
        ref, rstep, rpad = orc.film_grid(w, h, grain, ts)
        assert (step, pad) == (rstep, rpad), (w, h, grain, ts)
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            assert (a.idx, a.tx, a.ty, a.x_start, a.y_start, a.tw, a.th) == \
                (b.idx, b.tx, b.ty, b.x_start, b.y_start, b.tw, b.th)
        # The windows cover the image.
        cover = np.zeros((h, w), np.uint8)
        for t in got:
            cover[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw] = 1
        assert cover.all()


def test_tile_seeds_equal_the_oracle():
    tiles, _, _ = im.tile_grid(4096, 2731, 1.1)
    rtiles, _, _ = orc.film_grid(4096, 2731, 1.1, 320)
    for seed in SEEDS:
        for a, b in zip(tiles, rtiles):
            assert im.tile_seed(seed, a) == orc.film_tile_seed(seed, b)
