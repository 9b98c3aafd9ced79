"""GPU tests of the tile pipeline: device synthesis, the plain per-tile path and the batched
graph path, against each other and against the CPU oracle."""
import numpy as np
import pytest

import fgrain_gb300 as fg
from oracle import oracle as orc
from tests.helpers import reference_cfg, tile_cfg

pytestmark = pytest.mark.gpu


def ramp(h, w):
    return np.tile(np.linspace(0.0, 1.0, w, dtype=np.float32), (h, 1))


MIXED = [("tri-x", 1 / 2.4, 64, 48, 1.0, 0.0, 11), ("t-max", 1 / 1.1, 40, 40, 0.8, 1.0, 12),
         ("hp5", 1 / 1.8, 50, 30, 1.3, 0.5, 13), ("tri-x", 1 / 2.2, 33, 70, 0.6, 2.0, 14)]


def mixed_tiles():
    params = [fg.tile_params(*m) for m in MIXED]
    rng = np.random.default_rng(5)
    tiles = [rng.random((p.height_px, p.width_px)).astype(np.float32) for p in params]
    return params, tiles


def test_batch_equals_plain_path(engine):
    params, tiles = mixed_tiles()
    plain = [fg.render_tile(t, p, engine) for t, p in zip(tiles, params)]
    for use_graph, autotune in ((False, False), (True, False), (True, True)):
        b = fg.Batch(params, engine, use_graph=use_graph, autotune=autotune)
        b.set_exposure(tiles)
        for _ in range(2):  # replays give the same result
            b.run()
            st = b.wait()
            out = b.density()
            for o, q in zip(out, plain):
                np.testing.assert_array_equal(o, q)
        assert st["graph"] == int(use_graph)
        b.close()
    for q in plain:
        assert np.isfinite(q).all() and (q >= 0.05 - 1e-6).all() and (q <= 4.05 + 1e-5).all()


def test_synthesis_is_hard_core_at_bridson_density(engine):
    from scipy.spatial import cKDTree

    p = fg.tile_params("tri-x", 1 / 2.4, 256, 256, 1.0, 0.0, 0)
    b = fg.Batch([p], engine)
    b.set_exposure([ramp(256, 256)])
    b.run()
    b.wait()
    c = b.tile_crystals(0)
    pos = c["pos"]
    n = len(pos)
    W, H, D, r = p.film_w, p.film_h, p.film_d, p.r_min
    assert (pos >= 0).all() and (pos[:, 0] < W).all() and (pos[:, 1] < H).all() and (pos[:, 2] < D).all()
    d, _ = cKDTree(pos).query(pos, k=2)
    assert d[:, 1].min() >= r * (1 - 1e-6)
    # Count: the Bridson density model for this box, within binomial thinning noise.
    target = (0.57793168 + 0.11306788 * r * (2 / W + 2 / H + 2 / D)) / r ** 3 * W * H * D
    assert abs(n - target) < 4 * np.sqrt(target * 0.01) + 2
    # ... and the oracle's Bridson on the same box.
    ref = np.mean([len(orc.sample_poisson((W, H, D), r, 30, s)) for s in range(2)])
    assert abs(n - ref) / ref < 0.004
    # Attributes (emulsion.rs:162-184): radius clamp, cube dims, sensitivity floor, unit quats.
    rad = c["dims"][:, 0]
    assert rad.min() >= 0.15 - 1e-7 and rad.max() <= 0.48 * r + 1e-6
    assert np.allclose(c["dims"][:, 1], rad) and np.allclose(c["dims"][:, 2], rad)
    assert (c["sensitivity"] >= 0.1 - 1e-7).all()
    assert np.allclose(np.linalg.norm(c["quat"], axis=1), 1.0, atol=1e-5)
    orc_cr = orc.synthesize(reference_cfg("tri-x", W, H), 0)
    assert abs(np.mean(rad) - np.mean(orc_cr.dims[:, 0])) < 4 * np.std(rad) / np.sqrt(n)
    assert abs(np.mean(c["sensitivity"]) - np.mean(orc_cr.sens)) < 4 * 0.15 / np.sqrt(n)
    # Depth profile has no layering beyond Bridson's (cell grid period 3 cells).
    h, _ = np.histogram(pos[:, 2], bins=28, range=(0, D))
    assert h[2:-2].std() / h[2:-2].mean() < 0.05


def test_tabular_synthesis(engine):
    p = fg.tile_params("t-max", 1 / 1.1, 96, 96, 1.0, 0.0, 3)
    b = fg.Batch([p], engine)
    b.set_exposure([ramp(96, 96)])
    b.run()
    b.wait()
    c = b.tile_crystals(0)
    rad, ht = c["dims"][:, 0], c["dims"][:, 2]
    assert np.allclose(ht, np.maximum(rad / 6.5, 0.05), rtol=1e-6)
    tilt = 2 * np.arccos(np.clip(c["quat"][:, 3], -1, 1))
    assert tilt.max() <= 0.17 + 1e-5 and (np.abs(c["quat"][:, 2]) < 1e-7).all()
    assert (c["morphology"] == 1).all()


@pytest.mark.parametrize("stock,grain,expo,push", [("tri-x", 2.4, 1.0, 0.0), ("t-max", 1.1, 3.0, 2.0),
                                                   ("hp5", 1.8, 1.0, 2.0)])
def test_pipeline_matches_oracle_on_the_same_crystals(engine, stock, grain, expo, push):
    """The device's own synthesized crystals pushed through the oracle's expose / develop / scan
    reproduce the device tile: counts and the developed mask nearly everywhere, density to 1e-5.
    Each stock with its own tile-worker settings (exposure multiplier, push)."""
    p = fg.tile_params(stock, 1 / grain, 96, 80, expo, push, 21)
    tile = ramp(80, 96)
    b = fg.Batch([p], engine)
    b.set_exposure([tile])
    b.run()
    st = b.wait()
    d_dev = b.density()[0]
    c = b.tile_crystals(0)
    cfg = tile_cfg(p)
    dcfg = fg.DevelopmentConfig(p.threshold_photons, p.filament_expansion, p.clumping_proximity_factor, 0.85)
    cr = orc.Crystals(c["pos"], c["dims"], c["quat"], c["sensitivity"], c["morphology"])
    # The batch's development totals against the oracle's development of the device's own counts.
    crd = cr.copy()
    crd.latent[:] = c["counts"]
    rd = orc.develop(crd, dcfg)
    assert st["developed"] == int(c["developed"].sum()) == rd["developed_crystals"] > 100
    assert st["clumps"] == rd["total_clumps"]
    np.testing.assert_array_equal(crd.developed, c["developed"])
    np.testing.assert_allclose(crd.expansion, c["expansion"], rtol=1e-6)
    ecfg = fg.ExposureConfig(p.photons_per_sq_um * max(expo, 0.05), p.illumination_angle_rad,
                             p.crystal_absorption_coeff, p.max_bounces)
    orc.expose(cr, cfg, tile, ecfg, p.seed + 1, orc.FAITHFUL)
    same = (cr.latent == c["counts"]).mean()
    assert same > 0.99, same
    orc.develop(cr, dcfg)
    # Scan the device's developed mask with the oracle: isolates the scan stage.
    cr2 = cr.copy()
    cr2.developed[:] = c["developed"]
    cr2.expansion[:] = c["expansion"]
    r = orc.scan(cr2, cfg, fg.ScanConfig(96, 80, p.samples_per_pixel, 0, p.silver_opacity), p.seed + 2)
    T_orc = np.clip(r["T64"], 1e-4, 1.0)  # the density conversion clamps T (image_pipeline.rs:1009)
    d_orc = (-np.log10(T_orc) + 0.05).astype(np.float32)
    T_dev = 10.0 ** (-(d_dev.astype(np.float64) - 0.05))
    assert (np.abs(T_dev - T_orc) / T_orc).max() < 2e-5
    assert np.abs(d_dev - d_orc).max() < 1e-5
    assert (cr.developed == c["developed"]).mean() > 0.995


def test_statistical_parity_with_oracle_renders(engine):
    """Mean transmittance and grain noise power of whole device tiles (device Bridson columns,
    FP32 transport) against the oracle's tiles (sequential Bridson, FP64 transport) over seeds."""
    px, tw, th = 1 / 2.4, 112, 112
    flat = np.full((th, tw), 0.55, np.float32)
    seeds = list(range(100, 112))
    dev, orcs = [], []
    params = [fg.tile_params("tri-x", px, tw, th, 1.0, 0.0, s) for s in seeds]
    b = fg.Batch(params, engine)
    b.set_exposure([flat] * len(seeds))
    b.run()
    b.wait()
    for d_dev, s in zip(b.density(), seeds):
        d_orc, _ = orc.render_tile("tri-x", px, flat, 1.0, 0.0, s, orc.FAITHFUL)
        dev.append(d_dev)
        orcs.append(d_orc)
    dev, orcs = np.array(dev, np.float64), np.array(orcs, np.float64)
    Td, To = 10 ** (-(dev - 0.05)), 10 ** (-(orcs - 0.05))
    for name, fd, fo in (("mean T", Td.mean(axis=(1, 2)), To.mean(axis=(1, 2))),
                         ("noise power", dev.var(axis=(1, 2)), orcs.var(axis=(1, 2)))):
        diff = fd.mean() - fo.mean()
        sig = np.sqrt(fd.var(ddof=1) / len(fd) + fo.var(ddof=1) / len(fo))
        assert abs(diff) <= 3 * sig, (name, fd.mean(), fo.mean(), sig)


def radial_psd_bands(img, bands=((0.03, 0.1), (0.1, 0.2), (0.2, 0.35), (0.35, 0.5))):
    """Radially averaged power spectrum of a tile's density fluctuation, averaged per band of
    spatial frequency (cycles per pixel)."""
    f = np.fft.fft2(img - img.mean())
    p = np.abs(f) ** 2 / img.size
    k = np.hypot(np.fft.fftfreq(img.shape[0])[:, None], np.fft.fftfreq(img.shape[1])[None, :])
    return np.array([p[(k >= lo) & (k < hi)].mean() for lo, hi in bands])


def test_grain_noise_power_spectrum_matches_oracle(engine):
    """The grain's radially averaged noise power spectrum, band by band, agrees with the oracle's
    tiles within 3 sigma over 16 seeds (flat exposure, so the spectrum is the grain's alone)."""
    px, tw, th = 1 / 2.4, 96, 96
    flat = np.full((th, tw), 0.5, np.float32)
    seeds = list(range(300, 316))
    params = [fg.tile_params("tri-x", px, tw, th, 1.0, 0.0, s) for s in seeds]
    b = fg.Batch(params, engine)
    b.set_exposure([flat] * len(seeds))
    b.run()
    b.wait()
    dev = np.array([radial_psd_bands(d.astype(np.float64)) for d in b.density()])
    orcs = np.array([radial_psd_bands(orc.render_tile("tri-x", px, flat, 1.0, 0.0, s, orc.FAITHFUL)[0]
                                      .astype(np.float64)) for s in seeds])
    for j in range(dev.shape[1]):
        diff = dev[:, j].mean() - orcs[:, j].mean()
        sig = np.sqrt(dev[:, j].var(ddof=1) / len(seeds) + orcs[:, j].var(ddof=1) / len(seeds))
        assert abs(diff) <= 3 * sig, (j, dev[:, j].mean(), orcs[:, j].mean(), sig)


def test_identical_tiles_in_one_batch_stay_identical(engine):
    """Copies of one tile share warps in the transport (the photon queue interleaves tiles at its
    boundaries) and hit crystals with the same local indices: every copy must still get exactly
    its own counts, so all copies equal the plain render."""
    p = fg.tile_params("tri-x", 1 / 2.4, 96, 96, 1.0, 0.0, 77)
    tile = np.random.default_rng(77).random((96, 96)).astype(np.float32)
    plain = fg.render_tile(tile, p, engine)
    b = fg.Batch([p] * 12, engine)
    b.set_exposure([tile] * 12)
    b.run()
    b.wait()
    for d in b.density():
        np.testing.assert_array_equal(d, plain)
    b.close()
