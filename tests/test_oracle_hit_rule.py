"""How far the canonical hit rule (a crystal counts when its geometry and its own max_dim box are
hit, hits absorbed in t_enter order) is from the reference's own rule (the oracle's FAITHFUL mode:
every crystal of every reached leaf counts by its geometry, hits absorbed in traversal order,
bvh.rs:300-347, transport.rs:108-138), on the photon segments of configuration C1 and of one C2
tile.  The device follows the reference's rule; these numbers record why it must: the canonical
rule drops a fifth of the hits and reorders a third of the segments.  Also pins the tile grid and
seeds of the image driver against the oracle's restatement (image_pipeline.rs:377-434)."""
import numpy as np
import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import image as im
from oracle import oracle as orc
from tests.helpers import blurred_noise, reference_cfg, tile_worker_exposure_cfg


def c1_case():
    px = 1.0 / 2.4
    cfg = reference_cfg("tri-x", 256 * px, 256 * px)
    tile = np.tile(np.linspace(0.0, 1.0, 256, dtype=np.float32), (256, 1))
    return cfg, orc.synthesize(cfg, 0), tile, tile_worker_exposure_cfg(1.0), 1


def c2_tile_case():
    """Tile 24 (the centre) of configuration C2's 7 x 7 grid, with C2's exposure."""
    from scipy.ndimage import zoom

    lum = blurred_noise(1024, 1024, 16.0, 1, gamma=2.2).astype(np.float64)
    exposure = zoom(lum, 2, order=1, mode="nearest").astype(np.float32)
    grid, _, _ = im.tile_grid(2048, 2048, 2.4)
    t = grid[24]
    px = 1.0 / 2.4
    cfg = reference_cfg("tri-x", t.tw * px, t.th * px)
    seed = im.tile_seed(42, t)
    tile = np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw])
    return cfg, orc.synthesize(cfg, seed), tile, tile_worker_exposure_cfg(1.0), seed + 1


@pytest.mark.parametrize("case", [c1_case, c2_tile_case])
def test_canonical_rule_differs_from_the_reference_rule(case):
    cfg, cr, tile, ecfg, seed = case()
    r = orc.hit_rule_difference(cr, cfg, tile, ecfg, seed)
    print(case.__name__, r)
    assert r["segments"] > 50000
    # Every canonical hit is a reference hit (own box inside leaf box); the reference adds the
    # corner hits of rotated cubes that stick out of their own box but lie inside the leaf box.
    assert r["segments_canonical_not_subset"] == 0
    assert r["hits_faithful"] > r["hits_canonical"]
    assert 0.05 < r["hits_rel_diff"] < 0.5
    assert r["segments_hit_set_differs"] > 0.1 and r["segments_order_differs"] > 0.05
    # The absorbed energy moves far less than the hit count: corner chords are short.
    assert abs(r["latent_rel_diff"]) < 0.05


@pytest.mark.parametrize("w,h,grain,tile", [(1024, 768, 2.4, 320), (2048, 2048, 2.4, 320), (16384, 16384, 1.1, 320),
                                            (300, 7, 1.8, 64), (1, 1, 2.2, 320), (5000, 3000, 0.05, 320)])
def test_tile_grid_and_seeds_match_the_oracle(w, h, grain, tile):
    grid, step, pad = im.tile_grid(w, h, grain, tile)
    ogrid, ostep, opad = orc.film_grid(w, h, grain, tile)
    assert (step, pad) == (ostep, opad) and len(grid) == len(ogrid)
    for a, b in zip(grid, ogrid):
        assert (a.idx, a.tx, a.ty, a.x_start, a.y_start, a.tw, a.th) == (b.idx, b.tx, b.ty, b.x_start, b.y_start,
                                                                          b.tw, b.th)
        for s in (0, 42, 2**64 - 5):
            assert im.tile_seed(s, a) == orc.film_tile_seed(s, b)
