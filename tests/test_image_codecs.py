"""JPEG and lossless WebP files of the command-line tool (the image crate's ``jpeg`` and ``webp``
features behind image::open / ImageBuffer::save, src/image_pipeline.rs:1087-1152, Cargo.toml:13),
coded by the library's host C++ (``fg_jpeg_*``, ``fg_webp_*``; no GPU involved).

WebP is lossless: every encoder tool (each transform, pixel bundling, colour cache, meta prefix
codes, backward references with short and long distances) must give the pixels back exactly.
JPEG is lossy: round trips are held to PSNR floors that rise with quality, constant images come
back exact, and the decoder reads real-world files written by another encoder (scikit-learn's
sample photographs, when installed) without block-edge artefacts.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from fgrain_gb300 import _abi, imageio

RNG = np.random.default_rng(2024)
W = _abi
SINGLE_TOOLS = [W.FG_WEBP_SUBTRACT_GREEN, W.FG_WEBP_PREDICTOR, W.FG_WEBP_COLOR_TRANSFORM, W.FG_WEBP_PALETTE,
                W.FG_WEBP_COLOR_CACHE, W.FG_WEBP_BACKREFS, W.FG_WEBP_META_CODES,
                W.FG_WEBP_PREDICTOR | W.FG_WEBP_ALL_MODES]
OPTION_SETS = [0, W.FG_WEBP_DEFAULT, 0xFF] + SINGLE_TOOLS


def smooth(h, w, ch):
    y, x = np.mgrid[0:h, 0:w]
    planes = [(x * 3 + y * 2) % 256, (x * 5 + 17) % 256, (y * 7 + x) % 256, 255 - (x + y) % 64]
    img = np.stack(planes[:max(ch, 1)], -1).astype(np.uint8)
    return img[:, :, 0] if ch == 1 else img


def psnr(a, b):
    d = a.astype(np.float64) - b.astype(np.float64)
    m = (d * d).mean()
    return 99.0 if m == 0 else 10 * np.log10(255.0 ** 2 / m)


def as_rgba(img):
    if img.ndim == 2:
        img = np.repeat(img[:, :, None], 3, axis=2)
    if img.shape[2] == 3:
        img = np.concatenate([img, np.full(img.shape[:2] + (1,), 255, np.uint8)], axis=2)
    return img


# ---- WebP ----

@pytest.mark.parametrize("shape", [(1, 1), (1, 17), (13, 1), (7, 13), (33, 48), (64, 64)])
@pytest.mark.parametrize("ch", [1, 3, 4])
def test_webp_lossless_round_trip_every_tool(shape, ch):
    imgs = [smooth(*shape, ch), RNG.integers(0, 256, shape + ((ch,) if ch > 1 else ()), dtype=np.uint8)]
    for img in imgs:
        for opt in OPTION_SETS:
            got = imageio.decode_webp_rgba(imageio.encode_webp(img, opt))
            np.testing.assert_array_equal(got, as_rgba(img), err_msg=f"options {opt:#x}")


@pytest.mark.parametrize("ncolours", [1, 2, 3, 4, 5, 16, 17, 200, 256, 257])
def test_webp_colour_indexing_bundles(ncolours):
    """Palettes of <= 2, <= 4, <= 16 colours pack 8, 4, 2 pixels per bundled pixel; more than 256
    colours fall back to direct coding."""
    pal = RNG.integers(0, 256, (ncolours, 4), dtype=np.uint8)
    pal[:, 3] = np.where(np.arange(ncolours) % 3 == 0, 255, pal[:, 3])
    for w in (1, 5, 9, 31):
        idx = RNG.integers(0, ncolours, (11, w))
        img = pal[idx]
        for opt in (W.FG_WEBP_PALETTE, W.FG_WEBP_PALETTE | W.FG_WEBP_DEFAULT, 0xFF):
            got = imageio.decode_webp_rgba(imageio.encode_webp(img, opt))
            np.testing.assert_array_equal(got, img, err_msg=f"width {w} options {opt:#x}")


def test_webp_backward_references_short_and_long_distances():
    """Rows that repeat the row above (the short distance code for (0, 1)), the pixel 130 rows up
    (a plain distance), and runs longer than one length symbol covers."""
    w = 37
    base = RNG.integers(0, 256, (150, w, 3), dtype=np.uint8)
    base[1::2] = base[0::2]  # each odd row repeats the row above
    base[140:] = base[10:20]  # 130 rows up
    flat = np.zeros((40, 300, 3), np.uint8)  # 12,000 equal pixels: lengths up to 4096
    for img in (base, flat):
        for opt in (W.FG_WEBP_BACKREFS, W.FG_WEBP_BACKREFS | W.FG_WEBP_COLOR_CACHE, W.FG_WEBP_DEFAULT, 0xFF):
            data = imageio.encode_webp(img, opt)
            np.testing.assert_array_equal(imageio.decode_webp(data), img)
    assert len(imageio.encode_webp(flat, W.FG_WEBP_BACKREFS)) < 200


def test_webp_files_read_as_rgb_and_write_lossless(tmp_path):
    """image::open of a WebP gives Rgb8/Rgba8, which the renderer takes through to_rgb8; saving
    writes lossless WebP, so gray comes back replicated into RGB, exactly."""
    g = smooth(29, 41, 1)
    rgb = RNG.integers(0, 256, (23, 19, 3), dtype=np.uint8)
    imageio.write_image(tmp_path / "g.webp", g)
    imageio.write_image(tmp_path / "c.WEBP", rgb)
    np.testing.assert_array_equal(imageio.read_image(tmp_path / "g.webp"), np.repeat(g[:, :, None], 3, axis=2))
    np.testing.assert_array_equal(imageio.read_image(tmp_path / "c.WEBP"), rgb)
    rgba = RNG.integers(0, 256, (5, 6, 4), dtype=np.uint8)
    (tmp_path / "a.webp").write_bytes(imageio.encode_webp(rgba))
    np.testing.assert_array_equal(imageio.read_image(tmp_path / "a.webp"), rgba[:, :, :3])
    data = (tmp_path / "g.webp").read_bytes()
    assert data[:4] == b"RIFF" and data[8:16] == b"WEBPVP8L" and int.from_bytes(data[4:8], "little") == len(data) - 8


def riff(chunks):
    body = b"WEBP" + b"".join(k + len(v).to_bytes(4, "little") + v + b"\0" * (len(v) & 1) for k, v in chunks)
    return b"RIFF" + len(body).to_bytes(4, "little") + body


def test_webp_unsupported_and_corrupt_files_raise():
    good = imageio.encode_webp(smooth(16, 16, 3))
    vp8l = good[20:20 + int.from_bytes(good[16:20], "little")]
    cases = {
        "lossy": riff([(b"VP8 ", b"\x00" * 30)]),
        "animated": riff([(b"VP8X", b"\x02" + b"\x00" * 9), (b"ANIM", b"\x00" * 6)]),
        "signature": riff([(b"VP8L", b"\x2e" + vp8l[1:])]),
        "version": riff([(b"VP8L", vp8l[:4] + bytes([vp8l[4] | 0x20]) + vp8l[5:])]),
        "truncated": riff([(b"VP8L", vp8l[:len(vp8l) // 2])]),
        "no image": riff([(b"EXIF", b"abc")]),
        "not riff": b"RIFX" + good[4:],
    }
    for name, data in cases.items():
        with pytest.raises(imageio.ImageFormatError):
            imageio.decode_webp_rgba(data)
    with pytest.raises(imageio.ImageFormatError, match="lossy"):
        imageio.decode_webp_rgba(cases["lossy"])
    with pytest.raises(imageio.ImageFormatError):
        imageio.encode_webp(np.zeros((16385, 1), np.uint8))


def test_webp_info_reports_size_and_alpha_hint():
    lib = _abi.load()
    for img, alpha in ((smooth(9, 300, 3), 0), (smooth(9, 300, 4), 1)):
        data = imageio.encode_webp(img)
        w, h, a = C.c_uint32(), C.c_uint32(), C.c_uint32()
        assert lib.fg_webp_info(data, len(data), C.byref(w), C.byref(h), C.byref(a), None, 0) == 0
        assert (w.value, h.value, a.value) == (300, 9, alpha)


# ---- JPEG ----

def gradient(h, w, ch):
    """Ramps and a slanted wave without wrap-around (sharp 255 -> 0 steps in a chroma plane would
    measure the 2x2 chroma subsampling rather than the coding)."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    planes = [40 + 180 * x / max(w - 1, 1), 30 + 200 * y / max(h - 1, 1), 128 + 90 * np.sin((x + 2 * y) / 9.0)]
    img = np.rint(np.stack(planes[:ch], -1)).astype(np.uint8)
    return img[:, :, 0] if ch == 1 else img


# PSNR floors (dB) by quality; colour is bounded by the 2x2 chroma subsampling of the encoder.
JPEG_FLOORS = {1: {10: 30.0, 50: 40.0, 75: 43.0, 95: 50.0, 100: 60.0},
               3: {10: 24.0, 50: 29.0, 75: 31.0, 95: 34.0, 100: 34.0}}


@pytest.mark.parametrize("shape", [(1, 1), (7, 13), (17, 9), (16, 16), (75, 100), (300, 401)])
@pytest.mark.parametrize("ch", [1, 3])
def test_jpeg_round_trip_quality_floors(shape, ch):
    img = gradient(*shape, ch)
    floors = JPEG_FLOORS[ch]
    last = 0.0
    for q, floor in floors.items():
        data = imageio.encode_jpeg(img, q)
        got = imageio.decode_jpeg(data)
        assert got.shape == img.shape
        p = psnr(got, img)
        assert p >= floor, (q, p)
        assert p >= last - 1.0  # quality buys fidelity
        last = p


@pytest.mark.parametrize("shape", [(1, 1), (9, 17), (16, 32), (41, 23), (70, 95)])
@pytest.mark.parametrize("sub", [W.FG_JPEG_SUBSAMPLE_420, W.FG_JPEG_SUBSAMPLE_422, W.FG_JPEG_SUBSAMPLE_444])
def test_jpeg_scan_layouts_and_restart_markers_decode_identically(shape, sub):
    """The decoder's paths for files this encoder does not write by default: 4:2:2 and 4:4:4
    sampling, one scan per component (whose blocks cover only the component, not the MCU grid)
    and restart intervals.  The same quantised coefficients in another layout must decode to
    the same pixels."""
    for ch in (1, 3):
        img = gradient(*shape, ch)
        base = imageio.decode_jpeg(imageio.encode_jpeg(img, 80, sub))
        assert psnr(base, img) > (40.0 if ch == 1 else 28.0)
        for extra in (W.FG_JPEG_SEPARATE_SCANS, W.FG_JPEG_RESTART(1), W.FG_JPEG_RESTART(3),
                      W.FG_JPEG_SEPARATE_SCANS | W.FG_JPEG_RESTART(2), W.FG_JPEG_RESTART(64)):
            data = imageio.encode_jpeg(img, 80, sub | extra)
            np.testing.assert_array_equal(imageio.decode_jpeg(data), base, err_msg=f"options {sub | extra:#x}")
            if extra == W.FG_JPEG_RESTART(1) and shape != (1, 1):  # more than one MCU
                assert b"\xff\xdd" in data and b"\xff\xd0" in data
            if extra & W.FG_JPEG_SEPARATE_SCANS and ch == 3:
                assert data.count(b"\xff\xda") == 3


def test_jpeg_full_chroma_beats_subsampled_colour():
    img = gradient(64, 80, 3)
    p = {sub: psnr(imageio.decode_jpeg(imageio.encode_jpeg(img, 95, sub)), img)
         for sub in (W.FG_JPEG_SUBSAMPLE_420, W.FG_JPEG_SUBSAMPLE_422, W.FG_JPEG_SUBSAMPLE_444)}
    assert p[W.FG_JPEG_SUBSAMPLE_444] > p[W.FG_JPEG_SUBSAMPLE_422] > p[W.FG_JPEG_SUBSAMPLE_420]
    assert p[W.FG_JPEG_SUBSAMPLE_444] > 45.0


def test_jpeg_constant_images_come_back_exact():
    for v in (0, 1, 77, 128, 200, 255):
        g = np.full((19, 23), v, np.uint8)
        assert np.abs(imageio.decode_jpeg(imageio.encode_jpeg(g)).astype(int) - v).max() == 0
        c = np.zeros((19, 23, 3), np.uint8) + np.array([v, 255 - v, 128], np.uint8)
        assert np.abs(imageio.decode_jpeg(imageio.encode_jpeg(c, 90)).astype(int) - c).max() <= 2


def test_jpeg_files_read_gray_as_gray_and_write_quality_75(tmp_path):
    """The crate's JPEG decoder gives L8 for a gray file (kept gray by the renderer) and Rgb8 for
    colour; ImageBuffer::save writes JpegEncoder's default quality, 75."""
    g = smooth(31, 17, 1)
    rgb = smooth(8, 33, 3)
    imageio.write_image(tmp_path / "g.jpg", g)
    imageio.write_image(tmp_path / "c.jpeg", rgb)
    assert imageio.read_image(tmp_path / "g.jpg").shape == (31, 17)
    assert imageio.read_image(tmp_path / "c.jpeg").shape == (8, 33, 3)
    assert (tmp_path / "g.jpg").read_bytes() == imageio.encode_jpeg(g, 75)
    assert (tmp_path / "c.jpeg").read_bytes() == imageio.encode_jpeg(rgb, 75)
    lib = _abi.load()
    data = (tmp_path / "c.jpeg").read_bytes()
    w, h, ch = C.c_uint32(), C.c_uint32(), C.c_uint32()
    assert lib.fg_jpeg_info(data, len(data), C.byref(w), C.byref(h), C.byref(ch), None, 0) == 0
    assert (w.value, h.value, ch.value) == (33, 8, 3)


def sof_patched(data, marker=None, precision=None):
    i = data.index(b"\xff\xc0")
    out = bytearray(data)
    if marker is not None:
        out[i + 1] = marker
    if precision is not None:
        out[i + 4] = precision
    return bytes(out)


def test_jpeg_unsupported_and_corrupt_files_raise():
    good = imageio.encode_jpeg(smooth(20, 20, 3))
    with pytest.raises(imageio.ImageFormatError, match="(?i)progressive"):
        imageio.decode_jpeg(sof_patched(good, marker=0xC2))
    for marker in (0xC3, 0xC9, 0xCA):  # lossless, arithmetic coding
        with pytest.raises(imageio.ImageFormatError):
            imageio.decode_jpeg(sof_patched(good, marker=marker))
    with pytest.raises(imageio.ImageFormatError):
        imageio.decode_jpeg(sof_patched(good, precision=12))
    for cut in (4, 30, len(good) // 2):
        with pytest.raises(imageio.ImageFormatError):
            imageio.decode_jpeg(good[:cut])
    with pytest.raises(imageio.ImageFormatError):
        imageio.decode_jpeg(b"\xff\xd8\xff\xe0")
    with pytest.raises(ValueError):
        imageio.encode_jpeg(smooth(8, 8, 1), 0)
    with pytest.raises(imageio.ImageFormatError):  # 3 is no subsampling mode
        imageio.encode_jpeg(smooth(8, 8, 3), 75, 3)


def sample_photos():
    try:
        import sklearn
    except ImportError:
        return []
    root = Path(sklearn.__file__).parent / "datasets" / "images"
    return [p for p in (root / "china.jpg", root / "flower.jpg") if p.exists()]


@pytest.mark.parametrize("path", sample_photos() or [pytest.param(None, marks=pytest.mark.skip("no sample JPEGs"))])
def test_jpeg_reads_photographs_written_by_another_encoder(path):
    """Files from a widely used encoder (JFIF, 4:2:0 or 4:4:4, its own Huffman tables): decoded
    without block-edge artefacts (a misread stream shows steps at every 8th column), and a
    quality-95 re-encode of the decoded photograph stays close to it."""
    img = imageio.read_image(path)
    assert img.shape == (427, 640, 3)
    g = np.abs(np.diff(img.astype(np.float64), axis=1)).mean(axis=(0, 2))
    edges, inner = g[7::8].mean(), np.delete(g, np.s_[7::8]).mean()
    assert edges < 1.25 * inner
    again = imageio.decode_jpeg(imageio.encode_jpeg(img, 95))
    assert psnr(again, img) > 35.0


def test_corrupt_files_decode_or_raise():
    """Bit flips, truncations and overwritten runs in JPEG and WebP files: the decoders return an
    image or raise ImageFormatError, never crash (a command line reads whatever file it is given)."""
    rng = np.random.default_rng(7)
    img = smooth(37, 53, 3)
    bases = [("j", imageio.encode_jpeg(img, 75)), ("j", imageio.encode_jpeg(img[:, :, 0], 50)),
             ("j", imageio.encode_jpeg(img, 90, W.FG_JPEG_SUBSAMPLE_422 | W.FG_JPEG_SEPARATE_SCANS | W.FG_JPEG_RESTART(2))),
             ("w", imageio.encode_webp(img, 0xFF)), ("w", imageio.encode_webp(img, W.FG_WEBP_DEFAULT)),
             ("w", imageio.encode_webp(img, 0))]
    decoded = 0
    for it in range(1200):
        kind, base = bases[it % len(bases)]
        b = bytearray(base)
        m = rng.integers(0, 3)
        if m == 0:
            for _ in range(rng.integers(1, 8)):
                i = rng.integers(0, len(b))
                b[i] ^= 1 << int(rng.integers(0, 8))
        elif m == 1:
            b = b[:rng.integers(0, len(b))]
        else:
            i = rng.integers(0, len(b))
            j = min(len(b), i + int(rng.integers(1, 64)))
            b[i:j] = rng.integers(0, 256, j - i).astype(np.uint8).tobytes()
        try:
            out = imageio.decode_jpeg(bytes(b)) if kind == "j" else imageio.decode_webp_rgba(bytes(b))
            assert out.dtype == np.uint8 and out.size > 0
            decoded += 1
        except imageio.ImageFormatError:
            pass
    assert 0 < decoded < 1200
