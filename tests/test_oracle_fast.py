"""CPU tests of the oracle's restatement of the reference's wgpu tile model (gpu.rs:491-938 and
the poisson / develop / scan shaders): grid set-up, closed-form cases and the model's
properties."""
import numpy as np
import pytest

from fgrain_gb300 import fast
from oracle import oracle as orc


def params(preset="tri-x", px=1 / 2.4, tw=48, th=40, exposure=1.0, push=0.0, seed=3):
    return fast.tile_params_fast(preset, px, tw, th, exposure, push, seed)


def test_grid_follows_gpu_rs():
    (w, h, d), cs = orc.fast_grid(params(tw=64, th=64))
    assert cs == np.float32(1.2) and (w, h) == (23, 23) and d == 12  # ceil(26.67 / 1.2), ceil(14 / 1.2)
    (w, h, d), cs = orc.fast_grid(params("t-max", tw=64, th=64))
    assert cs == 1.0 and d == 8  # cell max(r_min, 1) = 1 um; 8 um deep
    # More than 512 cells along x: the cell grows so that the larger side has 512 cells.
    (w, h, d), cs = orc.fast_grid(params(px=2.0, tw=384, th=100))
    assert w == 512 and h <= 512 and cs > 1.2 and d == int(np.ceil(np.float32(14.0) / np.float32(cs)))


def test_preset_table_matches_gpu_branch():
    p = params("hp5", push=1.0)
    assert (p.film_d, p.silver_opacity, p.r_min, p.mean_crystal_radius, p.size_variance, p.morphology) == \
        (12.5, 0.22, 1.1, 0.50, 0.30, 2)
    assert abs(p.filament_expansion - 1.20) < 1e-12 and abs(p.clumping_proximity_factor - 1.22) < 1e-12
    q = params("tri-x", push=2.0)  # the GPU branch keeps tri-x at push 2 (no 1600 emulsion)
    assert q.r_min == 1.2 and q.base_sensitivity == 1.2 and abs(q.filament_expansion - 1.32) < 1e-12


def test_dark_tile_dissolves_every_crystal():
    p = params()
    d, cells = orc.fast_tile(p, np.zeros((p.height_px, p.width_px), np.float32))
    assert (cells["flags"][..., 0] == 0).all() and (cells["flags"][..., 2] == 0).all()
    assert (d == np.float32(0.05)).all()


def test_shadow_cut_below_irradiance_005():
    p = params()
    d, cells = orc.fast_tile(p, np.full((p.height_px, p.width_px), 0.049, np.float32))
    assert (cells["flags"][..., 0] == 0).all()
    d, cells = orc.fast_tile(p, np.full((p.height_px, p.width_px), 0.8, np.float32))
    assert cells["flags"][..., 2].sum() > 0 and d.max() > 0.05


@pytest.mark.parametrize("preset", ["tri-x", "t-max", "hp5"])
def test_cells_are_well_formed(preset):
    p = params(preset)
    _, cells = orc.fast_tile(p, np.full((p.height_px, p.width_px), 0.7, np.float32))
    q = cells["rot"]
    np.testing.assert_allclose((q.astype(np.float64) ** 2).sum(-1), 1.0, atol=1e-5)
    (w, h, d), cs = orc.fast_grid(p)
    pos = cells["pos"]
    assert (pos[..., 0] >= 0).all() and (pos[..., 0] <= p.film_w + 1e-4).all()
    assert (pos[..., 2] >= 0).all() and (pos[..., 2] <= p.film_d + 1e-4).all()
    assert (cells["flags"][..., 1] == p.morphology).all()
    dev = cells["flags"][..., 2] == 1
    assert (cells["dims_exp"][..., 3][~dev] == 0).all()
    assert (cells["dims_exp"][..., 3][dev] >= np.float32(p.filament_expansion) - 1e-6).all()


def test_density_rises_with_exposure():
    p = params(tw=64, th=32)
    ramp = np.tile(np.linspace(0, 1, 64, dtype=np.float32), (32, 1))
    d, _ = orc.fast_tile(p, ramp)
    cols = d.mean(axis=0)
    assert cols[:8].mean() < 0.1 and cols[-8:].mean() > cols[24:32].mean() > cols[:8].mean()


def test_bright_tile_takes_the_gaussian_branch():
    """Expected counts above 30 use the normal approximation (develop.wgsl:110-116)."""
    p = params(exposure=20.0)
    _, cells = orc.fast_tile(p, np.ones((p.height_px, p.width_px), np.float32))
    assert cells["flags"][..., 3].max() > 40
