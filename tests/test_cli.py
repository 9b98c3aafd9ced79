"""The command line and its image files, without a GPU: the reference's own CLI tests
(src/main.rs:1022-1089) and PNG decoding of every colour type, bit depth, row filter and the
Adam7 interlace, against PNGs written here with a separate encoder."""
import io
import struct
import zlib

import numpy as np
import pytest

from fgrain_gb300 import cli, imageio


def run(*args):
    out = io.StringIO()
    cli.run_cli(["fgrain", *args], out=out)
    return out.getvalue()


def test_help_flags():
    """main.rs:1026-1046."""
    for args in [(), ("-h",), ("--help",), ("help",), ("help", "apply"), ("help", "gradient"), ("help", "tri-x"),
                 ("help", "t-max"), ("help", "halation"), ("help", "demo"), ("apply", "-h"), ("apply", "--help"),
                 ("gradient", "-h"), ("tri-x", "-h"), ("t-max", "-h"), ("halation", "-h"), ("demo", "-h"),
                 ("test.png", "-h")]:
        assert run(*args)


def err(*args):
    with pytest.raises(cli.CliError) as e:
        run(*args)
    return str(e.value)


def test_invalid_commands_and_options():
    """main.rs:1049-1078."""
    assert "unrecognized command 'unknown_command'" in err("unknown_command")
    assert "unrecognized option '--unknown_opt'" in err("--unknown_opt")
    assert "unknown help topic 'unknown_topic'" in err("help", "unknown_topic")
    assert "missing required argument" in err("apply")
    assert "unrecognized option '--unknown_flag'" in err("apply", "test.png", "--unknown_flag")
    assert "option '--preset' requires an argument" in err("apply", "test.png", "--preset")
    assert "invalid value 'not_a_number' for '--push'" in err("apply", "test.png", "--push", "not_a_number")
    assert "expected an integer (1-4)" in err("apply", "a.png", "--supersample", "x")
    assert "unexpected positional argument 'c.png'" in err("apply", "a.png", "b.png", "c.png")
    assert "unknown demo 'nope'" in err("demo", "nope")
    assert "unrecognized option '--x' for 'gradient'" in err("gradient", "--x")


def test_main_prints_error_and_exits_one(capsys):
    assert cli.main(["fgrain", "unknown_command"]) == 1
    assert capsys.readouterr().err.startswith("error: unrecognized command")
    assert cli.main(["fgrain", "--help"]) == 0


def test_is_image_file():
    """main.rs:1081-1089."""
    for p in ("photo.PNG", "scan.jpg", "sample.jpeg", "input.webp"):
        assert cli.is_image_file(p)
    for p in ("gradient", "apply", "tri-x"):
        assert not cli.is_image_file(p)


def opts(*args):
    return cli.apply_options(cli.parse_apply_args(["in.png", *args]), lambda *_: None)


def test_apply_defaults_follow_the_stock_and_format():
    """main.rs:478-527: push stocks, grain by stock and format, strength, eberhard, output size."""
    o = opts()
    assert (o.preset, o.grain_size_px, o.grain_strength, o.push, o.eberhard, o.seed) == ("tri-x", 2.4, 1.0, 0.0, 0.0, 42)
    assert o.scanner_otf and o.output_resolution is None and o.tile_size == 320 and o.supersample == 1
    o = opts("-p", "tri-x-1600")
    assert (o.push, o.grain_strength, o.grain_size_px) == (2.0, 1.25, 2.2)
    o = opts("-p", "caffenol", "--push", "0.5")
    assert (o.push, o.grain_strength, o.grain_size_px) == (0.5, 1.25, 2.2)
    o = opts("--push", "1.5")
    assert (o.grain_strength, o.grain_size_px) == (1.25, 2.2)
    assert opts("-p", "T-Max", "-f", "120").grain_size_px == pytest.approx(1.1 * 0.55)
    assert opts("-p", "hp5", "-f", "large").grain_size_px == pytest.approx(1.8 * 0.28)
    assert opts("--push", "-3").push == 0.0 and opts("--eberhard", "-1").eberhard == 0.0
    assert opts("-s", "0.01").grain_size_px == 0.05 and opts("-s", "6").grain_size_px == 6.0
    assert opts("--supersample", "9").supersample == 4 and opts("--supersample", "0").supersample == 1
    assert opts("-w", "640").output_resolution == (640, 0) and opts("--height", "480").output_resolution == (0, 480)
    assert opts("-w", "640", "--height", "480").output_resolution == (640, 480)
    o = opts("-c", "--no-scanner-otf", "--auto-scale", "--reference-res", "4000", "--scale", "1.5", "-e", "0.8",
             "--tile-size", "256", "--grain-strength", "0.7", "--gpu")
    assert o.color and not o.scanner_otf and o.auto_scale and o.reference_res == 4000
    assert (o.scale, o.exposure, o.tile_size, o.grain_strength) == (1.5, 0.8, 256, 0.7)
    s = cli.parse_apply_args(["a.png", "b.png"])
    assert (s["input"], s["output"]) == ("a.png", "b.png")
    assert cli.parse_apply_args(["a.png", "-o", "c.png"])["output"] == "c.png"


def test_demo_exposure_tiles():
    """The demos' exposure closures (main.rs:829-835, 914-926, 991) on their sampling grid."""
    for name in ("gradient", "halation", "tri-x", "t-max"):
        preset, size, res, *_rest = cli._demo_spec(name)
        fn = _rest[3]
        t = cli.demo_exposure_tile(fn, size)
        assert t.shape == (round(size / cli.DEMO_SAMPLE_UM),) * 2 and t.dtype == np.float32
        if name == "gradient":
            assert t[0, 0] == pytest.approx(0.02, abs=1e-3) and t[0, -1] == pytest.approx(1.0, abs=1e-2)
            assert np.all(np.diff(t[0]) > 0)
        elif name == "halation":
            assert t.max() == pytest.approx(1.2) and t.min() == pytest.approx(0.04)
            assert (t > 1).sum() == pytest.approx(np.pi * 4.0 ** 2 / cli.DEMO_SAMPLE_UM ** 2, rel=0.02)
        else:
            assert np.all(t == np.float32(0.45))


# ---- PNG files written by an encoder independent of fgrain_gb300.imageio ----

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _filter_rows(rows, bpp, types):
    """Applies PNG filter types[y] to each row of raw bytes (h, stride)."""
    r = rows.astype(np.int32)
    h, n = r.shape
    out = np.zeros((h, n + 1), np.uint8)
    for y in range(h):
        cur = r[y]
        up = r[y - 1] if y else np.zeros(n, np.int32)
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        ul = np.concatenate([np.zeros(bpp, np.int32), up[:-bpp]])
        t = types[y % len(types)]
        pred = [0 * cur, left, up, (left + up) // 2, _paeth(left, up, ul)][t]
        out[y, 0] = t
        out[y, 1:] = (cur - pred) & 0xFF
    return out


def _pack(samples, depth):
    """(h, w, spp) samples to raw scanline bytes."""
    h, w, spp = samples.shape
    if depth == 8:
        return samples.astype(np.uint8).reshape(h, -1)
    if depth == 16:
        return samples.astype(">u2").reshape(h, -1).view(np.uint8).reshape(h, -1)
    bits = ((samples.reshape(h, w * spp)[:, :, None] >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8)
    return np.packbits(bits.reshape(h, -1), axis=1)


def _png(samples, depth, ctype, types=(0,), interlace=False, palette=None, trns=None):
    h, w, spp = samples.shape
    bpp = max(1, spp * depth // 8)
    if interlace:
        parts = []
        for x0, y0, dx, dy in ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2),
                               (0, 1, 1, 2)):
            sub = samples[y0::dy, x0::dx]
            if sub.size:
                parts.append(_filter_rows(_pack(sub, depth), bpp, types).tobytes())
        raw = b"".join(parts)
    else:
        raw = _filter_rows(_pack(samples, depth), bpp, types).tobytes()

    def chunk(k, b):
        return struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b) & 0xFFFFFFFF)

    z = zlib.compress(raw)
    body = chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        body += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    if trns is not None:
        body += chunk(b"tRNS", trns)
    # IDAT split in two chunks, as encoders often do
    return imageio.PNG_SIGNATURE + body + chunk(b"IDAT", z[:len(z) // 2]) + chunk(b"IDAT", z[len(z) // 2:]) + \
        chunk(b"IEND", b"")


RNG = np.random.default_rng(5)


@pytest.mark.parametrize("interlace", [False, True])
@pytest.mark.parametrize("types", [(0,), (1,), (2,), (3,), (4,), (0, 1, 2, 3, 4)])
def test_png_gray8_and_rgb8_every_filter(types, interlace):
    g = RNG.integers(0, 256, (23, 37, 1))
    np.testing.assert_array_equal(imageio.decode_png(_png(g, 8, 0, types, interlace)), g[:, :, 0])
    rgb = RNG.integers(0, 256, (19, 13, 3))
    np.testing.assert_array_equal(imageio.decode_png(_png(rgb, 8, 2, types, interlace)), rgb)
    rgba = RNG.integers(0, 256, (9, 30, 4))
    np.testing.assert_array_equal(imageio.decode_png(_png(rgba, 8, 6, types, interlace)), rgba[:, :, :3])


@pytest.mark.parametrize("interlace", [False, True])
def test_png_sixteen_bit_and_alpha_go_to_rgb8(interlace):
    g16 = RNG.integers(0, 65536, (11, 17, 1))
    want = (g16[:, :, 0] + 128) // 257
    got = imageio.decode_png(_png(g16, 16, 0, (4, 3), interlace))
    assert got.shape == (11, 17, 3)  # not ImageLuma8: the renderer takes the RGB route
    np.testing.assert_array_equal(got, np.repeat(want[:, :, None], 3, axis=2))
    rgb16 = RNG.integers(0, 65536, (7, 5, 3))
    np.testing.assert_array_equal(imageio.decode_png(_png(rgb16, 16, 2, (1, 4), interlace)), (rgb16 + 128) // 257)
    ga = RNG.integers(0, 256, (6, 9, 2))
    np.testing.assert_array_equal(imageio.decode_png(_png(ga, 8, 4, (2,), interlace)),
                                  np.repeat(ga[:, :, :1], 3, axis=2))


@pytest.mark.parametrize("depth", [1, 2, 4])
@pytest.mark.parametrize("interlace", [False, True])
def test_png_low_bit_depths(depth, interlace):
    g = RNG.integers(0, 1 << depth, (13, 21, 1))
    got = imageio.decode_png(_png(g, depth, 0, (0, 1, 4), interlace))
    np.testing.assert_array_equal(got, g[:, :, 0] * (255 // ((1 << depth) - 1)))
    pal = RNG.integers(0, 256, (1 << depth, 3))
    got = imageio.decode_png(_png(g, depth, 3, (2, 3), interlace, palette=pal))
    np.testing.assert_array_equal(got, pal[g[:, :, 0]])


def test_png_gray_with_transparency_takes_the_rgb_route():
    g = RNG.integers(0, 256, (5, 6, 1))
    got = imageio.decode_png(_png(g, 8, 0, trns=b"\x00\x07"))
    np.testing.assert_array_equal(got, np.repeat(g, 3, axis=2))


def test_png_one_pixel_and_bad_files():
    np.testing.assert_array_equal(imageio.decode_png(_png(np.array([[[200]]]), 8, 0, (4,), True)), [[200]])
    good = _png(RNG.integers(0, 256, (4, 4, 1)), 8, 0)
    bad = bytearray(good)
    bad[-20] ^= 0xFF  # inside the last IDAT: its CRC no longer matches
    with pytest.raises(imageio.ImageFormatError):
        imageio.decode_png(bytes(bad))
    with pytest.raises(imageio.ImageFormatError):
        imageio.decode_png(good[:40])


def test_writers_round_trip(tmp_path):
    g = RNG.integers(0, 256, (31, 17)).astype(np.uint8)
    rgb = RNG.integers(0, 256, (8, 33, 3)).astype(np.uint8)
    for name, img in (("a.png", g), ("b.png", rgb), ("c.pgm", g), ("d.ppm", rgb)):
        imageio.write_image(tmp_path / name, img)
        np.testing.assert_array_equal(imageio.read_image(tmp_path / name), img)
    imageio.write_image(tmp_path / "f.webp", rgb)  # lossless
    np.testing.assert_array_equal(imageio.read_image(tmp_path / "f.webp"), rgb)
    imageio.write_image(tmp_path / "e.jpg", g)  # lossy: same shape, gray stays gray
    assert imageio.read_image(tmp_path / "e.jpg").shape == g.shape
    (tmp_path / "g.jpg").write_bytes(b"\xff\xd8\xff\xe0")
    with pytest.raises(imageio.ImageFormatError):
        imageio.read_image(tmp_path / "g.jpg")
    (tmp_path / "i.gif").write_bytes(b"GIF89a")
    with pytest.raises(imageio.ImageFormatError, match="not a PNG, JPEG, WebP"):
        imageio.read_image(tmp_path / "i.gif")
    (tmp_path / "h.pgm").write_bytes(b"P5\n# comment\n2 2\n65535\n" + np.array([0, 65535, 257, 32896], ">u2").tobytes())
    np.testing.assert_array_equal(imageio.read_image(tmp_path / "h.pgm"), [[0, 255], [1, 128]])
