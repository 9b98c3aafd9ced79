"""GPU tests of the film renderer around the tile path: each stage against the oracle on the same
inputs (luma, resize and PSF bit for bit; the finishing stage on the device's own tile densities,
within one output level), the whole renderer against the composition of its stages, and the
reference's own image tests (image_pipeline.rs:1158-1326) on the device renderer."""
import numpy as np
import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import film
from fgrain_gb300 import image as im
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("preset", ["tri-x", "hp5", "t-max", "ektar"])
def test_luma_bit_exact(engine, preset):
    rgb = np.random.default_rng(1).integers(0, 256, (61, 83, 3), dtype=np.uint8)
    np.testing.assert_array_equal(film.panchromatic_luma(rgb, preset, engine), orc.luma(rgb, preset))


@pytest.mark.parametrize("filt", [film.TRIANGLE, film.LANCZOS3])
@pytest.mark.parametrize("shape", [(64, 64, 32, 32), (50, 70, 123, 97), (300, 200, 75, 50), (13, 7, 13, 29),
                                   (1, 40, 3, 9), (64, 48, 64, 48)])
def test_resize_bit_exact(engine, filt, shape):
    h, w, oh, ow = shape
    img = np.random.default_rng(h + w).integers(0, 256, (h, w), dtype=np.uint8)
    np.testing.assert_array_equal(film.resize_u8(img, ow, oh, filt, engine), orc.resize_u8(img, ow, oh, filt))


def psf_cases():
    rng = np.random.default_rng(2)
    a = rng.integers(0, 256, (70, 90), dtype=np.uint8)
    b = a.copy()
    b[:9] = 0
    b[-5:] = 0
    b[:, :3] = 0
    b[30:40, 40:60] = 0
    c = np.zeros((20, 20), np.uint8)
    d = np.zeros((33, 17), np.uint8)
    d[16, 8] = 5
    return [a, b, c, d]


@pytest.mark.parametrize("k", range(4))
def test_gelatin_psf_bit_exact(engine, k):
    img = psf_cases()[k]
    h, g = film.gelatin_psf(img, engine)
    ho, go = orc.gelatin_psf(img)
    assert g == go
    np.testing.assert_array_equal(h, ho)


def device_tiles(src, heff, preset, grain, push, seed, tile_size, engine):
    H, W = src.shape
    grid, step, pad = im.tile_grid(W, H, grain, tile_size)
    params = im.image_tile_params(preset, grain, grid, 1.0, push, seed)
    tiles = [np.ascontiguousarray(heff[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]) for t in grid]
    return grid, step, pad, im.render_tiles(params, tiles, engine)


@pytest.mark.parametrize("preset,grain,push,otf", [("tri-x", 2.4, 0.0, True), ("t-max", 1.1, 1.5, True),
                                                   ("hp5", 1.8, 0.0, False)])
def test_finish_against_oracle_on_device_tiles(engine, preset, grain, push, otf):
    rng = np.random.default_rng(4)
    from scipy.ndimage import gaussian_filter
    src = (np.clip(gaussian_filter(rng.random((180, 260)), 6) * 4 - 1.5, 0, 1) * 255).astype(np.uint8)
    src[:10] = 0
    heff, _ = film.gelatin_psf(src, engine)
    grid, step, pad, dens = device_tiles(src, heff, preset, grain, push, 7, 96, engine)
    H, W = src.shape
    out, st, fl = film.film_finish(preset, grain, 1.0, push, otf, W, H, grid, step, pad, dens, src, heff, True, engine)
    oo, so, flo = orc.film_finish(preset, grain, 1.0, push, otf, W, H, grid, step, pad, dens, src, heff, True)
    # d_norm: the Hann cosine is correctly rounded on the device, the C library's cosf in the oracle.
    np.testing.assert_allclose(fl[0], flo[0], rtol=2e-7, atol=1e-7)
    np.testing.assert_allclose(fl[1], flo[1], rtol=0, atol=1e-6)
    # Grain statistics: FP64 tree sums on the device, sequential f32 sums in the oracle.
    np.testing.assert_allclose(st[:3], so[:3], rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(fl[3], flo[3], rtol=0, atol=1e-6)
    # Grain and scanned grain carry the statistics' difference (relative) and the composite's
    # powf / sinf rounding (absolute).
    np.testing.assert_allclose(fl[2], flo[2], rtol=2e-4, atol=2e-6)
    np.testing.assert_allclose(fl[4], flo[4], rtol=2e-4, atol=2e-6)
    d = np.abs(out.astype(int) - oo.astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())


def compose_bw(gray, opts, engine):
    """The renderer's stages called one by one (image_pipeline.rs:299-891)."""
    h, w = gray.shape
    ow, oh = opts.output_resolution or (w, h)
    ss = opts.supersample
    rw, rh = ow * ss, oh * ss
    src = film.resize_u8(gray, rw, rh, film.LANCZOS3, engine)
    heff, _ = film.gelatin_psf(src, engine)
    grain = opts.grain_size_px
    grid, step, pad, dens = device_tiles(src, heff, opts.preset, grain, opts.push, opts.seed, opts.tile_size, engine)
    out, _ = film.film_finish(opts.preset, grain, opts.grain_strength, opts.push, opts.scanner_otf, rw, rh, grid, step,
                              pad, dens, src, heff, False, engine)
    return out if ss == 1 else film.resize_u8(out, ow, oh, film.TRIANGLE, engine)


def test_render_equals_its_stages(engine):
    gray = np.random.default_rng(5).integers(0, 256, (150, 210), dtype=np.uint8)
    opts = film.FilmRenderOptions(preset="tri-x", grain_size_px=2.4, tile_size=64, seed=9)
    rep, out = film.render_film(gray, opts, engine)
    assert rep.output_resolution == (210, 150) and rep.total_tiles == 4 * 3
    np.testing.assert_array_equal(out, compose_bw(gray, opts, engine))


def test_render_resized_and_supersampled_equals_its_stages(engine):
    gray = np.random.default_rng(6).integers(0, 256, (90, 120), dtype=np.uint8)
    opts = film.FilmRenderOptions(preset="hp5", grain_size_px=1.8, tile_size=96, seed=3, supersample=2,
                                  output_resolution=(100, 75))
    rep, out = film.render_film(gray, opts, engine)
    assert out.shape == (75, 100)
    np.testing.assert_array_equal(out, compose_bw(gray, opts, engine))


def test_rgb_gray_render_is_render_of_its_luma(engine):
    rgb = np.random.default_rng(7).integers(0, 256, (64, 80, 3), dtype=np.uint8)
    opts = film.FilmRenderOptions(preset="t-max", grain_size_px=1.1, tile_size=64)
    _, a = film.render_film(rgb, opts, engine)
    _, b = film.render_film(film.panchromatic_luma(rgb, "t-max", engine), opts, engine)
    np.testing.assert_array_equal(a, b)


def test_color_render_is_three_layers_with_offset_seeds(engine):
    """render_film_color_tiled (image_pipeline.rs:1017-1085), also the reference's 48x48 colour
    pipeline test (image_pipeline.rs:1197-1231) without the file round trip."""
    rgb = np.array([[(x * 5, y * 5, 128) for x in range(48)] for y in range(48)], np.uint8)
    opts = film.FilmRenderOptions(tile_size=48, grain_size_px=2.0)
    rep, out = film.render_film_color_tiled(rgb, opts, engine)
    assert out.shape == (48, 48, 3) and rep.input_resolution == (48, 48)
    for c, off in enumerate(im.COLOR_SEED_OFFSETS):
        o = film.FilmRenderOptions(tile_size=48, grain_size_px=2.0, seed=42 + off)
        _, layer = film.render_film(np.ascontiguousarray(rgb[..., c]), o, engine)
        np.testing.assert_array_equal(out[..., c], layer)


def test_color_render_against_the_oracle_driver(engine):
    """The oracle's restatement of the colour driver (channel split, the three seed offsets,
    interleave; image_pipeline.rs:1017-1085) and of the whole renderer, fed with tile densities the
    device renders for exactly the tiles and seeds that driver asks for, against fg_render_film's
    colour output: equal within one output level on under 1 % of pixels (the finish's statistics
    are FP64 tree sums on the device, sequential f32 sums in the oracle)."""
    rng = np.random.default_rng(12)
    from scipy.ndimage import gaussian_filter
    rgb = np.stack([(np.clip(gaussian_filter(rng.random((96, 120)), 5) * 3 - 1, 0, 1) * 255).astype(np.uint8)
                    for _ in range(3)], -1)
    kw = dict(preset="hp5", grain_size_px=1.8, tile_size=64, seed=5, supersample=2, output_resolution=(100, 80))
    opts = film.FilmRenderOptions(color=True, **kw)
    _, out = film.render_film(rgb, opts, engine)

    def tile_fn(preset, grain, exposure, push, jobs):
        params = [fg.tile_params(preset, 1.0 / grain, t.shape[1], t.shape[0], exposure, push, s) for s, t in jobs]
        return im.render_tiles(params, [t for _, t in jobs], engine)

    ref = orc.film_render_color(rgb, tile_fn=tile_fn, **kw)
    assert out.shape == ref.shape == (80, 100, 3)
    d = np.abs(out.astype(int) - ref.astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 0.01, (d.max(), (d > 0).mean())
    assert (out[..., 0] != out[..., 1]).mean() > 0.3  # the layers are independent renders


def test_reference_gray_pipeline_dimensions(engine):
    """image_pipeline.rs:1158-1195 without the file round trip."""
    g = np.array([[(x + y) * 2 for x in range(64)] for y in range(64)], np.uint8)
    rep, out = film.render_film_black_and_white_tiled(g, film.FilmRenderOptions(tile_size=64, grain_size_px=2.0),
                                                       engine)
    assert rep.input_resolution == (64, 64) and rep.output_resolution == (64, 64) and out.shape == (64, 64)


@pytest.mark.parametrize("size", [2.4, 10.0, 20.0])
def test_reference_letterbox_and_shadow_zero_variance(engine, size):
    """image_pipeline.rs:1233-1280 on the device renderer."""
    img = np.full((64, 64), 200, np.uint8)
    img[:8] = 0
    img[56:] = 0
    img[24:40, 24:40] = 0
    _, out = film.render_film(img, film.FilmRenderOptions(tile_size=64, grain_size_px=size, scanner_otf=True),
                              engine)
    assert (out[:8] == 0).all() and (out[56:] == 0).all() and (out[26:38, 26:38] == 0).all()


def test_reference_highlight_fusion_burnout(engine):
    """image_pipeline.rs:1282-1325 on the device renderer."""
    img = np.full((64, 64), 128, np.uint8)
    img[:, :32] = 255
    _, out = film.render_film(img, film.FilmRenderOptions(tile_size=64, grain_size_px=2.4), engine)
    fog = out[4:60, 4:28]
    assert fog.min() >= 253 and fog.max() == 255


def test_render_rejects_bad_arguments(engine):
    with pytest.raises(fg.GpuError):
        film.render_film(np.zeros((8, 8), np.uint8), film.FilmRenderOptions(tile_size=16), engine)
    with pytest.raises(ValueError):
        film.render_film(np.zeros((8, 8, 2), np.uint8), None, engine)


def test_render_in_several_batches_equals_one_batch(engine):
    """With a small device budget the tiles run as consecutive batches; tiles are independent, so
    the photograph is the same bit for bit."""
    rgb = np.random.default_rng(8).integers(0, 256, (200, 260, 3), dtype=np.uint8)
    opts = film.FilmRenderOptions(preset="hp5", grain_size_px=1.8, tile_size=64, color=True, seed=3)
    rep1, one = film.render_film(rgb, opts, engine)
    for budget in (64 << 20, 1):
        small = film.FilmRenderOptions(**{**opts.__dict__, "batch_bytes": budget})
        rep, many = film.render_film(rgb, small, engine)
        np.testing.assert_array_equal(one, many)
        assert rep.total_crystals == rep1.total_crystals and rep.total_tiles == rep1.total_tiles
        assert (rep.developed_crystals, rep.total_clumps) == (rep1.developed_crystals, rep1.total_clumps)
    assert 0 < rep1.total_clumps <= rep1.developed_crystals < rep1.total_crystals


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (5, 3), (49, 1)])
def test_tiny_and_ragged_images_render(engine, shape):
    """Images smaller than a tile, one pixel wide or one pixel high: one clipped tile each; the
    device renderer agrees with the composition of its stages and keeps the output size."""
    gray = np.random.default_rng(sum(shape)).integers(40, 256, shape, dtype=np.uint8)
    opts = film.FilmRenderOptions(preset="tri-x", grain_size_px=2.4, tile_size=64, seed=1)
    rep, out = film.render_film(gray, opts, engine)
    assert out.shape == shape and rep.total_tiles == 1
    np.testing.assert_array_equal(out, compose_bw(gray, opts, engine))


def test_all_black_photograph_stays_black(engine):
    """Zero exposure everywhere: the camera gate is empty, no grain, every output pixel 0
    (image_pipeline.rs:137-155 and the output gates, 866-882)."""
    _, out = film.render_film(np.zeros((70, 90, 3), np.uint8), film.FilmRenderOptions(color=True, tile_size=64), engine)
    assert (out == 0).all()
