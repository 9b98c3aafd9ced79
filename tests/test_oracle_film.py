"""CPU tests of the oracle's image stages (luma, the image crate's resampler, the gelatin PSF and
the finishing stage), each against an independent numpy restatement or a closed form, and the
reference's own image-pipeline tests (image_pipeline.rs:1158-1326) run through the oracle's
whole-image renderer."""
import numpy as np
import pytest

from oracle import oracle as orc

f32 = np.float32


def np_luma(rgb, w):
    r, g, b = (rgb[..., k].astype(f32) for k in range(3))
    v = (r * w[0] + g * w[1]) + b * w[2]
    v = np.clip(v, f32(0), f32(255))
    return np.floor(np.abs(v) + f32(0.5)).astype(np.uint8)  # round half away (v >= 0)


@pytest.mark.parametrize("preset", ["tri-x", "hp5", "t-max", "other"])
def test_luma_matches_numpy_float32(preset):
    rgb = np.random.default_rng(0).integers(0, 256, (37, 53, 3), dtype=np.uint8)
    w = orc.luma_weights(preset)
    np.testing.assert_array_equal(orc.luma(rgb, preset), np_luma(rgb, w))


def test_luma_weights_table():
    assert list(orc.luma_weights("Tri-X")) == list(np.array([0.42, 0.46, 0.12], f32))
    assert list(orc.luma_weights("caffenol")) == list(np.array([0.42, 0.46, 0.12], f32))
    assert list(orc.luma_weights("hp5-plus")) == list(np.array([0.36, 0.48, 0.16], f32))
    assert list(orc.luma_weights("tmax")) == list(np.array([0.33, 0.52, 0.15], f32))
    assert list(orc.luma_weights("ektar")) == list(np.array([0.38, 0.48, 0.14], f32))


def np_axis_weights(n, m, filt):
    ratio = f32(n) / f32(m)
    sratio = f32(1) if ratio < 1 else ratio
    support = (f32(1) if filt == orc.TRIANGLE else f32(3)) * sratio
    out = []
    for o in range(m):
        c = (f32(o) + f32(0.5)) * ratio
        left = min(max(int(np.floor(c - support)), 0), n - 1)
        right = min(max(int(np.ceil(c + support)), left + 1), n)
        c = c - f32(0.5)
        ws = []
        for i in range(left, right):
            x = (f32(i) - c) / sratio
            if filt == orc.TRIANGLE:
                v = f32(1) - abs(x) if abs(x) < 1 else f32(0)
            else:
                def sinc(t):
                    a = f32(t * f32(np.pi))
                    return f32(1) if t == 0 else f32(np.sin(np.float32(a), dtype=f32) / a)
                v = f32(sinc(x) * sinc(x / f32(3))) if abs(x) < 3 else f32(0)
            ws.append(f32(v))
        s = f32(0)
        for v in ws:
            s = f32(s + v)
        out.append((left, [f32(v / s) for v in ws]))
    return out


def np_resize(img, ow, oh, filt):
    h, w = img.shape
    if (ow, oh) == (w, h):
        return img.copy()
    tmp = np.zeros((oh, w), f32)
    for y, (l, ws) in enumerate(np_axis_weights(h, oh, filt)):
        t = np.zeros(w, f32)
        for i, v in enumerate(ws):
            t = t + img[l + i].astype(f32) * v
        tmp[y] = t
    out = np.zeros((oh, ow), np.uint8)
    for x, (l, ws) in enumerate(np_axis_weights(w, ow, filt)):
        t = np.zeros(oh, f32)
        for i, v in enumerate(ws):
            t = t + tmp[:, l + i] * v
        out[:, x] = np.floor(np.clip(t, 0, 255) + f32(0.5)).astype(np.uint8)
    return out


@pytest.mark.parametrize("filt", [orc.TRIANGLE, orc.LANCZOS3])
@pytest.mark.parametrize("shape", [(40, 30, 20, 15), (17, 23, 41, 29), (64, 64, 64, 64), (9, 50, 3, 7)])
def test_resize_matches_numpy_restatement(filt, shape):
    h, w, oh, ow = shape
    img = np.random.default_rng(h * w).integers(0, 256, (h, w), dtype=np.uint8)
    got = orc.resize_u8(img, ow, oh, filt)
    want = np_resize(img, ow, oh, filt)
    if filt == orc.TRIANGLE:
        np.testing.assert_array_equal(got, want)
    else:
        # numpy's float32 sin is not the C library's sinf: one level at a rounding boundary.
        assert np.abs(got.astype(int) - want.astype(int)).max() <= 1
        assert (got != want).mean() < 0.01


@pytest.mark.parametrize("filt", [orc.TRIANGLE, orc.LANCZOS3])
def test_resize_keeps_constant_images(filt):
    img = np.full((33, 47), 137, np.uint8)
    for ow, oh in [(20, 11), (90, 70), (47, 10)]:
        assert (orc.resize_u8(img, ow, oh, filt) == 137).all()


def test_psf_gate_and_uniform_interior():
    img = np.zeros((40, 50), np.uint8)
    img[6:31, 4:45] = 160
    img[15:20, 20:25] = 0  # a silhouette inside the gate is not part of the gate
    heff, gate = orc.gelatin_psf(img)
    assert gate == (6, 31, 4, 45)
    assert (heff[:6] == 0).all() and (heff[31:] == 0).all() and (heff[:, :4] == 0).all() and (heff[:, 45:] == 0).all()
    # Far from the silhouette the interior is uniform: the normalised taps give 160/255 to 1 ulp.
    np.testing.assert_allclose(heff[8:12, 6:16], np.float32(160) / np.float32(255), rtol=3e-7)
    assert heff[17, 22] < heff[8, 8]


def test_psf_of_empty_image_is_zero():
    heff, gate = orc.gelatin_psf(np.zeros((12, 9), np.uint8))
    assert gate == (12, 12, 9, 9) and (heff == 0).all()


def test_finish_of_flat_density_is_the_tone_curve():
    """d_norm constant -> d_high = 0, deviation clamps to 0.035, grain 0: the output is the tone."""
    W = H = 96
    grid, step, pad = orc.film_grid(W, H, 2.4, 64)
    dens = [np.full((t.th, t.tw), 0.7, np.float32) for t in grid]
    src = np.random.default_rng(3).integers(0, 256, (H, W), dtype=np.uint8)
    heff, _ = orc.gelatin_psf(src)
    out, st, fl = orc.film_finish("tri-x", 2.4, 1.0, 0.0, True, W, H, grid, step, pad, dens, src, heff, fields=True)
    np.testing.assert_allclose(fl[0], 0.7, rtol=1e-6)
    assert abs(st[0]) < 1e-6 and st[1] == np.float32(0.035)
    raw = src.astype(f32) / f32(255)
    base = np.where(raw <= f32(0.005), f32(0), f32(0.35) * raw + f32(0.65) * heff)
    want = np.floor(np.clip(base, 0, 1) * f32(255) + f32(0.5)).astype(np.uint8)
    np.testing.assert_array_equal(out, want)


def letterbox_image():
    img = np.full((64, 64), 200, np.uint8)
    img[:8] = 0
    img[56:] = 0
    img[24:40, 24:40] = 0
    return img


@pytest.mark.parametrize("size", [2.4, 10.0, 20.0])
def test_reference_letterbox_and_shadow_zero_variance(size):
    """image_pipeline.rs:1233-1280 through the oracle renderer."""
    out = orc.film_render_bw(letterbox_image(), tile_size=64, grain_size_px=size, scanner_otf=True)
    assert (out[:8] == 0).all() and (out[56:] == 0).all() and (out[26:38, 26:38] == 0).all()


def test_reference_highlight_fusion_burnout():
    """image_pipeline.rs:1282-1325 through the oracle renderer."""
    img = np.full((64, 64), 128, np.uint8)
    img[:, :32] = 255
    out = orc.film_render_bw(img, tile_size=64, grain_size_px=2.4)
    fog = out[4:60, 4:28]
    assert fog.min() >= 253 and fog.max() == 255


def test_reference_pipeline_dimensions():
    """image_pipeline.rs:1158-1231 (minus the file round trip): 64x64 gray and 48x48 colour."""
    g = np.array([[(x + y) * 2 for x in range(64)] for y in range(64)], np.uint8)
    assert orc.film_render_bw(g, tile_size=64, grain_size_px=2.0).shape == (64, 64)
    rgb = np.array([[(x * 5, y * 5, 128) for x in range(48)] for y in range(48)], np.uint8)
    layers = [orc.film_render_bw(rgb[..., c], tile_size=48, grain_size_px=2.0, seed=42 + off)
              for c, off in enumerate((0, 10007, 20011))]
    assert np.stack(layers, axis=-1).shape == (48, 48, 3)
