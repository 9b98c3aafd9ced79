"""The command line on the device: ``apply`` from a PNG file to a PNG file equals the renderer
called directly, and the demonstrations run through the engine entry points."""
import io

import numpy as np
import pytest

from fgrain_gb300 import cli, film, imageio

pytestmark = pytest.mark.gpu


def run(*args):
    out = io.StringIO()
    cli.run_cli(["fgrain", *args], out=out)
    return out.getvalue()


def test_apply_file_to_file_equals_render_film(tmp_path, engine):
    rng = np.random.default_rng(11)
    rgb = rng.integers(0, 256, (96, 128, 3), dtype=np.uint8)
    src, dst = tmp_path / "in.png", tmp_path / "out.png"
    imageio.write_image(src, rgb)
    text = run(str(src), str(dst), "-p", "hp5", "--tile-size", "64", "--supersample", "2")
    got = imageio.read_image(dst)
    opts = cli.apply_options(cli.parse_apply_args(["x", "-p", "hp5", "--tile-size", "64", "--supersample", "2"]),
                             lambda *_: None)
    rep, want = film.render_film(rgb, opts, engine)
    np.testing.assert_array_equal(got, want)
    assert f"Total Crystals:    {rep.total_crystals}" in text and "Silver Clumps:" in text
    assert rep.developed_crystals > 0 and f"Developed Silver:  {rep.developed_crystals}" in text


def test_apply_colour_to_ppm_and_missing_input(tmp_path, engine):
    g = np.random.default_rng(2).integers(0, 256, (40, 50), dtype=np.uint8)
    src = tmp_path / "g.pgm"
    imageio.write_image(src, g)
    run("apply", str(src), "-o", str(tmp_path / "c.ppm"), "-c", "-p", "t-max", "--tile-size", "48", "-w", "25")
    out = imageio.read_image(tmp_path / "c.ppm")
    assert out.shape == (20, 25, 3)
    with pytest.raises(cli.CliError, match="failed to process image"):
        run("apply", str(tmp_path / "missing.png"), str(tmp_path / "o.png"))


@pytest.mark.parametrize("name", ["gradient", "halation", "tri-x", "t-max"])
def test_demos(tmp_path, engine, name):
    dst = tmp_path / f"{name}.png"
    text = run("demo", name, str(dst))
    img = imageio.read_image(dst)
    res = 384 if name == "gradient" else 256
    assert img.shape == (res, res) and "Developed:" in text
    cols = img.astype(np.float64).mean(axis=0)
    # The positive print shows 1 - T (transmittance.rs:146): dense silver is bright.
    if name == "gradient":  # exposure rises along x (and development saturates in the highlights)
        bins = cols.reshape(8, -1).mean(axis=1)
        assert np.corrcoef(np.arange(res), cols)[0, 1] > 0.5 and bins[-1] > bins[0] + 10
    elif name == "halation":  # the intense core at the centre
        c = img[res // 2 - 8:res // 2 + 8, res // 2 - 8:res // 2 + 8].mean()
        assert c > img[:32, :32].mean()
    else:
        assert 0 < img.std()


@pytest.mark.parametrize("color", [False, True])
def test_webp_file_to_webp_file(tmp_path, engine, color):
    """src/image_pipeline.rs:1159-1229 (test_webp_read_write_pipeline, test_webp_color_pipeline):
    a WebP photograph (64 x 64 gray ramp, or 48 x 48 colour ramps) rendered with grain size 2 px
    and one tile to a WebP file, which loads back with the input's size.  WebP is lossless, so
    the file holds exactly the renderer's pixels (a gray render replicated into RGB)."""
    n = 48 if color else 64
    y, x = np.mgrid[0:n, 0:n]
    img = (np.stack([x * 5, y * 5, np.full_like(x, 128)], -1) if color else (x + y) * 2).astype(np.uint8)
    src, dst = tmp_path / "in.webp", tmp_path / "out.webp"
    imageio.write_image(src, img)
    args = ["--tile-size", str(n), "-s", "2.0"] + (["-c"] if color else [])
    run(str(src), str(dst), *args)
    got = imageio.read_image(dst)
    assert got.shape == (n, n, 3)
    opts = cli.apply_options(cli.parse_apply_args(["x", *args]), lambda *_: None)
    rep, want = film.render_film(imageio.read_image(src), opts, engine)
    assert rep.input_resolution == (n, n) and rep.output_resolution == (n, n)
    np.testing.assert_array_equal(got, want if color else np.repeat(want[:, :, None], 3, axis=2))


def test_jpeg_file_to_jpeg_file(tmp_path, engine):
    """A gray JPEG photograph rendered to a JPEG file: the output is the renderer's image of the
    decoded input, written at quality 75 (the image crate's default)."""
    y, x = np.mgrid[0:72, 0:88]
    img = (40 + x + y).astype(np.uint8)
    src, dst = tmp_path / "in.jpg", tmp_path / "out.jpg"
    imageio.write_image(src, img)
    run(str(src), str(dst), "--tile-size", "64", "-p", "t-max")
    opts = cli.apply_options(cli.parse_apply_args(["x", "--tile-size", "64", "-p", "t-max"]), lambda *_: None)
    _, want = film.render_film(imageio.read_image(src), opts, engine)
    assert dst.read_bytes() == imageio.encode_jpeg(want, 75)
    assert imageio.read_image(dst).shape == (72, 88)
