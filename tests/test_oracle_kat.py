"""The CPU oracle against the reference's own inline known-answer tests (CPU only).

Each test restates one #[test] of the reference crate with the same inputs and assertions,
citing it; a few derived analytic cases follow.  Philox is pinned to the Random123 vectors.
"""
import math

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import identity_quats, reference_cfg

import fgrain_gb300 as fg


def test_philox_known_answers():
    # Philox-4x32-10 known-answer vectors (Random123 kat_vectors).
    assert orc.philox((0, 0, 0, 0), (0, 0)) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert orc.philox((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert orc.philox((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_cubic_crystal_intersection():
    # crystal.rs:238-261
    hit = orc.intersect_crystal((10, 10, 10), (1, 1, 1), (0, 0, 0, 1), 0, 1.0, (10, 10, 0), (0, 0, 1))
    assert hit is not None
    assert abs(hit[0] - 9.0) < 1e-4 and abs(hit[1] - 11.0) < 1e-4
    assert orc.intersect_crystal((10, 10, 10), (1, 1, 1), (0, 0, 0, 1), 0, 1.0, (20, 10, 0), (0, 0, 1)) is None


def test_tabular_crystal_intersection():
    # crystal.rs:264-282
    hit = orc.intersect_crystal((0, 0, 5), (2, 2, 0.2), (0, 0, 0, 1), 1, 1.0, (0, 0, 0), (0, 0, 1))
    assert hit is not None
    assert abs(hit[0] - 4.8) < 1e-4 and abs(hit[1] - 5.2) < 1e-4


def _row_of_cubes(n, spacing, half, z):
    pos = np.array([[i * spacing, 0.0, z] for i in range(n)])
    return orc.Crystals(pos, np.full((n, 3), half), identity_quats(n), np.ones(n), np.zeros(n, np.int32))


@pytest.mark.parametrize("mode", [orc.FAITHFUL, orc.CANONICAL])
def test_bvh_construction_and_query(mode):
    # bvh.rs:412-439: 20 unit cubes on x = 3i, a ray at x = 15 hits exactly crystal 5.
    cr = _row_of_cubes(20, 3.0, 1.0, 10.0)
    nodes, depth = orc.bvh_stats(cr)
    assert nodes > 0
    idx, t0, t1 = orc.ray_hits(cr, (15, 0, 0), (0, 0, 1), mode)
    assert idx.tolist() == [5]


def test_bvh_radius_query():
    # bvh.rs:442-462
    cr = _row_of_cubes(10, 1.0, 0.4, 0.0)
    assert orc.query_radius(cr, (5, 0, 0), 1.5) == [4, 5, 6]


def test_poisson_min_distance():
    # poisson.rs:141-165 (20x20x10, r_min 2, k 30, seed 42): all pairs at least r_min - 1e-6 apart.
    pts = orc.sample_poisson((20.0, 20.0, 10.0), 2.0, 30, 42)
    assert len(pts) > 0
    d2 = ((pts[:, None, :] - pts[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    assert d2.min() >= (2.0 - 1e-6) ** 2
    assert (pts >= 0).all() and (pts[:, 0] < 20).all() and (pts[:, 1] < 20).all() and (pts[:, 2] < 10).all()


def test_emulsion_synthesis():
    # emulsion.rs:233-253 (t-max 25 x 25, seed 42): non-empty, centres inside the volume.
    cfg = reference_cfg("t-max", 25.0, 25.0)
    cr = orc.synthesize(cfg, 42)
    assert len(cr) > 0
    assert (cr.pos >= 0).all()
    assert (cr.pos[:, 0] <= 25).all() and (cr.pos[:, 1] <= 25).all() and (cr.pos[:, 2] <= 8).all()
    # Radius clamp [0.15, 0.48 r_min] and tabular thickness (emulsion.rs:169,187).
    r = cr.dims[:, 0]
    assert r.min() >= 0.15 and r.max() <= 0.48 * 0.9 + 1e-12
    assert np.allclose(cr.dims[:, 2], np.maximum(r / 6.5, 0.05))
    assert (cr.sens >= 0.1).all()
    assert np.allclose(np.linalg.norm(cr.quat, axis=1), 1.0)


def test_free_path_distribution():
    # optics.rs:206-224: mean free path within 5% of 1/mu_t over 10k draws.
    optics = fg.GelatinOptics()
    xs = [orc.free_path(optics, orc.philox((i, 0, 0, 0x4650), (123, 0))[0] / 2**32) for i in range(10000)]
    mfp = 1.0 / (optics.absorption_coeff + optics.scattering_coeff)
    assert abs(np.mean(xs) - mfp) / mfp < 0.05


def test_antihalation_energy_attenuation():
    # optics.rs:227-245: energy decreases, reflected direction points up (-z).
    optics = fg.GelatinOptics()
    for u in ([0.5, 0.1, 0.3, 0.7], [0.5, 0.9, 0.3, 0.7], [0.05, 0.2, 0.9, 0.1]):
        alive, E, d = orc.antihalation(optics, 1.0, (0.0, 0.0, 1.0), u)
        assert alive and E < 1.0 and d[2] < 0.0


def test_exposure_latent_image_formation():
    # transport.rs:195-237: tri-x 20 x 20 (seed 100), left half exposed (x <= 10): the left
    # counts exceed five times the right counts.  The closure becomes a 2-pixel tile [1, 0].
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    cr = orc.synthesize(cfg, 100)
    ecfg = fg.ExposureConfig(100.0, 0.1, 1.5, 32)
    tile = np.array([[1.0, 0.0]], np.float32)
    P, _, _ = orc.expose(cr, cfg, tile, ecfg, 42)
    assert P == round(400 * 100.0)
    left = cr.latent[cr.pos[:, 0] <= 9.0].sum()
    right = cr.latent[cr.pos[:, 0] >= 11.0].sum()
    assert left > 0
    assert left > right * 5


def test_boolean_thresholding_and_clumping():
    # development.rs:197-265
    pos = np.array([[0.0, 0, 5], [0.8, 0, 5], [1.6, 0, 5], [10.0, 0, 5], [20.0, 0, 5]])
    cr = orc.Crystals(pos, np.full((5, 3), 0.5), identity_quats(5), np.ones(5), np.zeros(5, np.int32))
    cr.latent[:] = [10, 10, 10, 4, 1]
    rep = orc.develop(cr, fg.DevelopmentConfig(3, 2.0, 1.5, 0.75))
    assert rep["developed_crystals"] == 4 and rep["fixed_crystals"] == 1
    assert cr.developed[4] == 0
    assert cr.clump[0] == cr.clump[1] == cr.clump[2]
    assert cr.clump[3] != cr.clump[0]
    assert rep["total_clumps"] == 2 and rep["max_clump_size"] == 3
    # Boost of a 3-crystal clump: 2.0 * (1.15 + 0.18 * 2); the isolated crystal keeps 2.0.
    assert cr.expansion[0] == 2.0 * (1.15 + 0.18 * 2) and cr.expansion[3] == 2.0 and cr.expansion[4] == 0.0


def _single_cube_emulsion(cfg, seed):
    cr = orc.synthesize(cfg, seed)
    cr.developed[:] = 0
    cr.developed[0] = 1
    cr.pos[0] = (5.0, 5.0, 4.0)
    cr.dims[0] = (2.0, 2.0, 1.0)
    cr.quat[0] = (0, 0, 0, 1)
    cr.morph[0] = 0
    cr.expansion[0] = 1.0
    return cr


def test_transmittance_evaluation():
    # transmittance.rs:181-221: one developed cube, 16 x 16 px, 4 spp, sigma 20.
    cfg = reference_cfg("t-max", 10.0, 10.0)
    cr = _single_cube_emulsion(cfg, 123)
    r = orc.scan(cr, cfg, fg.ScanConfig(16, 16, 4, fg.ScanMode.NegativeTransmittance, 20.0), 42)
    buf = r["out"].ravel()
    assert buf[8 * 16 + 8] < buf[0]
    assert buf[0] > 0.95


def test_single_cube_chord_is_exact():
    # Derived: an axis-aligned developed cube of half-size (2, 2, 1) has chord 2 * 1 for every
    # ray inside its footprint, so T = exp(-2 sigma) there; elsewhere T = 1.
    cfg = reference_cfg("t-max", 10.0, 10.0)
    cr = _single_cube_emulsion(cfg, 123)
    r = orc.scan(cr, cfg, fg.ScanConfig(20, 20, 4, fg.ScanMode.NegativeTransmittance, 0.5), 7)
    T = r["T64"]
    inside = T[7:13, 7:13]  # pixels 0.5 um wide, footprint x, y in (3, 7)
    assert np.allclose(inside, math.exp(-0.5 * 2.0), rtol=0, atol=1e-15)
    assert np.allclose(T[:5, :], 1.0) and np.allclose(T[:, 15:], 1.0)


def test_empty_and_zero_opacity():
    cfg = reference_cfg("tri-x", 6.0, 6.0)
    cr = orc.synthesize(cfg, 3)
    r = orc.scan(cr, cfg, fg.ScanConfig(8, 8, 4, fg.ScanMode.NegativeTransmittance, 0.25), 1)
    assert (r["out"] == 1.0).all()  # nothing developed
    cr.developed[:] = 1
    cr.expansion[:] = 1.2
    r = orc.scan(cr, cfg, fg.ScanConfig(8, 8, 4, fg.ScanMode.NegativeTransmittance, 0.0), 1)
    assert (r["out"] == 1.0).all()  # sigma 0


def test_strata_lie_in_their_quarters():
    cfg = reference_cfg("tri-x", 8.0, 8.0)
    o = orc.scan_ray_origins(cfg, fg.ScanConfig(4, 4, 4, 0, 0.25), 11).reshape(4, 4, 2, 2, 3)
    pw = 2.0
    for py in range(4):
        for px in range(4):
            for sy in range(2):
                for sx in range(2):
                    x, y, z = o[py, px, sy, sx]
                    assert px * pw + sx * pw / 2 <= x < px * pw + (sx + 1) * pw / 2
                    assert py * pw + sy * pw / 2 <= y < py * pw + (sy + 1) * pw / 2
                    assert z == 14.0 + 0.1


def test_faithful_and_canonical_hit_sets():
    # Canonical is a subset of faithful (own box inside the leaf box); ellipsoids agree exactly.
    for preset in ("tri-x", "t-max"):
        cfg = reference_cfg(preset, 12.0, 12.0)
        cr = orc.synthesize(cfg, 5)
        cr.developed[:] = 1
        cr.expansion[:] = 1.2
        rng = np.random.default_rng(0)
        o = np.column_stack([rng.uniform(0, 12, 4000), rng.uniform(0, 12, 4000), np.full(4000, cfg.dimensions[2] + 0.1)])
        d = np.tile([0.0, 0.0, -1.0], (4000, 1))
        of, idf, _ = orc.rays_hits(cr, o, d, orc.FAITHFUL, True)
        oc, idc, _ = orc.rays_hits(cr, o, d, orc.CANONICAL, True)
        for r in range(4000):
            f = set(idf[of[r]:of[r + 1]].tolist())
            c = set(idc[oc[r]:oc[r + 1]].tolist())
            assert c <= f
            if preset == "t-max":
                assert c == f
