"""GPU parity of the transport / develop / scan path against the CPU oracle.

Every test runs the CUDA library through the C ABI and checks it against oracle/ on the same
seeded inputs, with the reference's own hit rule (the oracle's FAITHFUL mode: its spatial-median
BVH, leaf-box reach and traversal order, bvh.rs:157-347):
  * the device builds exactly the reference's tree: the same index order, leaves and leaf boxes;
  * recorded photon segments replayed on the device give the oracle's hit index lists and latent
    counts bit for bit;
  * development of identical counts gives the same developed mask, clump ids and expansions;
  * with a fixed developed mask, the scanned transmittance is within 1e-5 relative of the
    oracle's FP64 value, and every scanner ray finds exactly the oracle's hit set;
  * the production (FP32) transport reproduces the oracle's counts up to rare rounding flips.
"""
import numpy as np
import pytest

import fgrain_gb300 as fg
from oracle import oracle as orc
from tests.helpers import identity_quats, reference_cfg, tile_worker_dev_cfg, tile_worker_exposure_cfg

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5  # scanned transmittance vs the FP64 oracle (relative)


def upload(cr: orc.Crystals, cfg, engine):
    return fg.VirtualEmulsionLayer.from_crystals(cfg, cr.pos, cr.dims, cr.quat, cr.sens, cr.morph, engine)


def ramp_tile(h, w):
    """Configuration C1's exposure: a horizontal ramp 0 -> 1."""
    return np.tile(np.linspace(0.0, 1.0, w, dtype=np.float32), (h, 1))


# ------------------------------------------------------------------------------------------------
# Device known-answer tests (the reference's inline tests, through the C ABI)

def test_device_cubic_and_tabular_intersection(engine):
    cfg = reference_cfg("tri-x", 30.0, 30.0)
    pos = np.array([[10.0, 10.0, 10.0], [0.0, 0.0, 5.0]])
    dims = np.array([[1.0, 1.0, 1.0], [2.0, 2.0, 0.2]])
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, pos, dims, identity_quats(2), np.ones(2),
                                               np.array([0, 1], np.int32), engine)
    off, ids, chord = fg.replay_rays(em, [[10, 10, 0], [20, 10, 0], [0, 0, 0]],
                                     [[0, 0, 1], [0, 0, 1], [0, 0, 1]], developed_only=False)
    assert ids[off[0]:off[1]].tolist() == [0] and abs(chord[0] - 2.0) < 1e-12  # t 9 -> 11
    assert off[2] - off[1] == 0
    assert ids[off[2]:off[3]].tolist() == [1] and abs(chord[2] - 0.4) < 1e-12  # t 4.8 -> 5.2


def test_device_bvh_ray_hits_crystal_5(engine):
    # bvh.rs:412-439
    cfg = reference_cfg("tri-x", 60.0, 10.0)
    pos = np.array([[3.0 * i, 0.0, 10.0] for i in range(20)])
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, pos, np.ones((20, 3)), identity_quats(20), np.ones(20),
                                               None, engine)
    off, ids, _ = fg.replay_rays(em, [[15.0, 0.0, 0.0]], [[0.0, 0.0, 1.0]], developed_only=False)
    assert ids.tolist() == [5]


def test_device_thresholding_and_clumping(engine):
    # development.rs:197-265
    cfg = reference_cfg("tri-x", 30.0, 10.0)
    pos = np.array([[0.0, 0, 5], [0.8, 0, 5], [1.6, 0, 5], [10.0, 0, 5], [20.0, 0, 5]])
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, pos, np.full((5, 3), 0.5), identity_quats(5), np.ones(5),
                                               None, engine)
    em.set_latent_counts([10, 10, 10, 4, 1])
    rep = fg.develop_emulsion(em, fg.DevelopmentConfig(3, 2.0, 1.5, 0.75))
    assert rep.developed_crystals == 4 and rep.fixed_crystals == 1
    assert rep.total_clumps == 2 and rep.max_clump_size == 3
    dv, cl, ex = em.development()
    assert dv.tolist() == [1, 1, 1, 1, 0]
    assert cl.tolist() == [0, 0, 0, 1, -1]
    assert ex.tolist() == [2.0 * (1.15 + 0.18 * 2)] * 3 + [2.0, 0.0]


def test_device_transmittance_evaluation(engine):
    # transmittance.rs:181-221, and against the oracle on the same crystals.
    cfg = reference_cfg("t-max", 10.0, 10.0)
    cr = orc.synthesize(cfg, 123)
    cr.developed[:] = 0
    cr.developed[0] = 1
    cr.pos[0] = (5.0, 5.0, 4.0)
    cr.dims[0] = (2.0, 2.0, 1.0)
    cr.quat[0] = (0, 0, 0, 1)
    cr.morph[0] = 0
    cr.expansion[0] = 1.0
    em = upload(cr, cfg, engine)
    em.set_development(cr.developed, cr.expansion)
    sc = fg.ScanConfig(16, 16, 4, fg.ScanMode.NegativeTransmittance, 20.0)
    buf, img = fg.scan_emulsion(em, sc, 42)
    b = buf.ravel()
    assert b[8 * 16 + 8] < b[0] and b[0] > 0.95
    ref = orc.scan(cr, cfg, sc, 42)
    np.testing.assert_allclose(buf, ref["T64"], rtol=T_RTOL, atol=0)
    assert (img == ref["image8"]).all()


# ------------------------------------------------------------------------------------------------
# The reference tree (bvh.rs:157-295) built on the device

@pytest.mark.parametrize("preset,size,seed", [("tri-x", (40.0, 36.0), 1), ("hp5", (30.0, 24.0), 2),
                                              ("t-max", (26.0, 22.0), 3), ("tri-x", (200.0, 180.0), 4)])
def test_device_reference_tree_equals_the_oracle(engine, preset, size, seed):
    """Index order, leaf ranges and FP64 leaf boxes of the device's tree equal the oracle's
    restatement of BVH::build, over all crystals and over the developed ones with their expansion."""
    cfg = reference_cfg(preset, *size)
    cr = orc.synthesize(cfg, seed)
    rng = np.random.default_rng(seed)
    cr.developed[:] = (rng.random(len(cr)) < 0.4).astype(np.uint8)
    cr.expansion[:] = np.where(cr.developed == 1, 1.2 * (1.0 + 0.18 * rng.integers(0, 4, len(cr))), 0.0)
    em = upload(cr, cfg, engine)
    em.set_development(cr.developed, cr.expansion)
    for dev_only in (False, True):
        order, leaves, boxes = fg.reference_tree(em, dev_only)
        ro, rl, rb = orc.bvh_export(cr, dev_only)
        np.testing.assert_array_equal(order, ro)
        k = np.argsort(rl[:, 0], kind="stable")
        np.testing.assert_array_equal(leaves, rl[k])
        np.testing.assert_array_equal(boxes, rb[k])
    assert len(cr) > 1000


@pytest.mark.parametrize("n", [1, 2, 4, 5, 6, 33, 200, 1024, 1025, 2100])
def test_device_reference_tree_small_and_degenerate_sets(engine, n):
    """Sets at the leaf size, at the edge of the per-block finish (1024 crystals), and with
    coincident centroids (the reference's degenerate-extent leaf, bvh.rs:230-239)."""
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    rng = np.random.default_rng(n)
    pos = rng.random((n, 3)) * [20.0, 20.0, 14.0]
    if n >= 31:
        pos[: n // 3] = pos[0]  # a third of the crystals share one centre
    dims = np.full((n, 3), 0.4) * (1.0 + rng.random((n, 1)))
    cr = orc.Crystals(pos, dims, identity_quats(n), np.ones(n), np.zeros(n, np.int32))
    em = upload(cr, cfg, engine)
    order, leaves, boxes = fg.reference_tree(em)
    ro, rl, rb = orc.bvh_export(cr)
    np.testing.assert_array_equal(order, ro)
    k = np.argsort(rl[:, 0], kind="stable")
    np.testing.assert_array_equal(leaves, rl[k])
    np.testing.assert_array_equal(boxes, rb[k])


# ------------------------------------------------------------------------------------------------
# Configuration C1: 256 x 256 ramp, tri-x cubic grains, 2.4 px grain (0.41667 um pixels), seed 0.

C1_PX = 1.0 / 2.4


@pytest.fixture(scope="module")
def c1():
    """Oracle run of the C1 tile: crystals, recorded segments, counts, development."""
    tw = th = 256
    cfg = reference_cfg("tri-x", tw * C1_PX, th * C1_PX)
    tile = ramp_tile(th, tw)
    cr = orc.synthesize(cfg, 0)
    ecfg = tile_worker_exposure_cfg(1.0)
    P, segs, hits = orc.expose(cr, cfg, tile, ecfg, 1, orc.FAITHFUL, record=True)
    counts = cr.latent.copy()
    dcr = cr.copy()
    rep = orc.develop(dcr, tile_worker_dev_cfg("tri-x"))
    return dict(cfg=cfg, tile=tile, cr=cr, ecfg=ecfg, P=P, segs=segs, hits=hits, counts=counts,
                dev=dcr, rep=rep)


def test_c1_replayed_hits_and_counts_bit_exact(engine, c1):
    em = upload(c1["cr"], c1["cfg"], engine)
    off, ids = fg.replay_segments(em, c1["ecfg"], 1, c1["segs"])
    ro, rids = orc.replay_segments(c1["cr"].copy(), c1["ecfg"], 1, c1["segs"])
    assert len(c1["segs"]) > 100000
    np.testing.assert_array_equal(off, ro)
    np.testing.assert_array_equal(ids, rids)
    np.testing.assert_array_equal(em.latent_counts(), c1["counts"])


def test_c1_developed_mask_bit_exact(engine, c1):
    em = upload(c1["cr"], c1["cfg"], engine)
    em.set_latent_counts(c1["counts"])
    rep = fg.develop_emulsion(em, tile_worker_dev_cfg("tri-x"))
    dv, cl, ex = em.development()
    d = c1["dev"]
    np.testing.assert_array_equal(dv, d.developed)
    np.testing.assert_array_equal(cl, d.clump)
    np.testing.assert_array_equal(ex, d.expansion)
    r = c1["rep"]
    assert (rep.total_crystals, rep.developed_crystals, rep.fixed_crystals, rep.total_clumps,
            rep.max_clump_size) == (r["total_crystals"], r["developed_crystals"], r["fixed_crystals"],
                                    r["total_clumps"], r["max_clump_size"])
    assert rep.developed_crystals > 1000 and rep.max_clump_size > 1


def test_c1_scan_fixed_mask_matches_fp64(engine, c1):
    d = c1["dev"]
    em = upload(d, c1["cfg"], engine)
    em.set_development(d.developed, d.expansion)
    sc = fg.ScanConfig(256, 256, 4, fg.ScanMode.NegativeTransmittance, 0.25)
    buf, _ = fg.scan_emulsion(em, sc, 2)
    ref = orc.scan(d, c1["cfg"], sc, 2, orc.FAITHFUL, want_hits=True)
    rel = np.abs(buf.astype(np.float64) - ref["T64"]) / ref["T64"]
    assert rel.max() <= T_RTOL, rel.max()
    assert abs(buf.mean() - ref["T64"].mean()) / ref["T64"].mean() < 1e-6
    np.testing.assert_array_equal(fg.scan_ray_hits(em, sc, 2), ref["ray_hits"])
    assert (buf < 0.999).mean() > 0.2  # the tile really carries silver


def test_c1_scan_rays_hit_sets_bit_exact(engine, c1):
    d = c1["dev"]
    em = upload(d, c1["cfg"], engine)
    em.set_development(d.developed, d.expansion)
    sc = fg.ScanConfig(128, 128, 4, 0, 0.25)
    o = orc.scan_ray_origins(c1["cfg"], sc, 9)
    dirs = np.tile([0.0, 0.0, -1.0], (len(o), 1))
    off, ids, chord = fg.replay_rays(em, o, dirs, developed_only=True)
    ro, rids, rchord = orc.rays_hits(d, o, dirs, orc.FAITHFUL, developed_only=True)
    np.testing.assert_array_equal(off, ro)
    np.testing.assert_array_equal(ids, rids)
    np.testing.assert_allclose(chord, rchord, rtol=1e-12, atol=1e-12)


def test_c1_production_transport_matches_oracle(engine, c1):
    em = upload(c1["cr"], c1["cfg"], engine)
    fg.expose_emulsion(em, c1["tile"], c1["ecfg"], 1)
    got = em.latent_counts().astype(np.int64)
    ref = c1["counts"].astype(np.int64)
    t = engine.timings()
    assert t["photons"] == c1["P"]
    same = (got == ref).mean()
    assert same > 0.99, same
    assert abs(got.sum() - ref.sum()) / ref.sum() < 5e-3


# ------------------------------------------------------------------------------------------------
# Other stocks, strata counts and edge cases

@pytest.mark.parametrize("preset", ["t-max", "hp5", "tri-x-1600"])
def test_other_stocks_replay_develop_scan(engine, preset):
    px = {"t-max": 1 / 1.1, "hp5": 1 / 1.8, "tri-x-1600": 1 / 2.2}[preset]
    tw, th = 96, 80
    cfg = reference_cfg(preset, tw * px, th * px)
    cr = orc.synthesize(cfg, 17)
    tile = ramp_tile(th, tw)
    ecfg = tile_worker_exposure_cfg(1.5)
    P, segs, _ = orc.expose(cr, cfg, tile, ecfg, 18, orc.FAITHFUL, record=True)
    em = upload(cr, cfg, engine)
    off, ids = fg.replay_segments(em, ecfg, 18, segs)
    ro, rids = orc.replay_segments(cr.copy(), ecfg, 18, segs)
    np.testing.assert_array_equal(ids, rids)
    np.testing.assert_array_equal(em.latent_counts(), cr.latent)
    base = preset if preset != "tri-x-1600" else "tri-x"
    dcfg = tile_worker_dev_cfg(base, 2.0 if preset == "tri-x-1600" else 0.0)
    fg.develop_emulsion(em, dcfg)
    d = cr.copy()
    orc.develop(d, dcfg)
    dv, cl, ex = em.development()
    np.testing.assert_array_equal(dv, d.developed)
    np.testing.assert_array_equal(cl, d.clump)
    np.testing.assert_array_equal(ex, d.expansion)
    for spp in (1, 4, 9, 16):
        sc = fg.ScanConfig(tw, th, spp, fg.ScanMode.NegativeTransmittance, 0.25)
        buf, _ = fg.scan_emulsion(em, sc, 19)
        ref = orc.scan(d, cfg, sc, 19, want_hits=True)
        assert (np.abs(buf - ref["T64"]) / ref["T64"]).max() <= T_RTOL
        np.testing.assert_array_equal(fg.scan_ray_hits(em, sc, 19), ref["ray_hits"])


@pytest.mark.parametrize("mode", [fg.ScanMode.PositivePrint, fg.ScanMode.OpticalDensity])
def test_scan_modes_and_8bit_image(engine, mode):
    cfg = reference_cfg("tri-x", 30.0, 30.0)
    cr = orc.synthesize(cfg, 4)
    rng = np.random.default_rng(1)
    cr.developed[:] = rng.random(len(cr)) < 0.5
    cr.expansion[:] = np.where(cr.developed == 1, 1.2 * 1.33, 0.0)
    em = upload(cr, cfg, engine)
    em.set_development(cr.developed, cr.expansion)
    sc = fg.ScanConfig(64, 64, 4, mode, 0.25)
    buf, img = fg.scan_emulsion(em, sc, 5)
    ref = orc.scan(cr, cfg, sc, 5)
    np.testing.assert_allclose(buf, ref["out"], rtol=1e-5, atol=1e-6)
    assert np.abs(img.astype(int) - ref["image8"].astype(int)).max() <= 1


def test_identity_orientations_take_the_fp64_path(engine):
    # Axis-aligned cubes give inverse directions of +-inf for vertical rays: every decision goes to
    # the FP64 path, which must still agree exactly.
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    cr = orc.synthesize(cfg, 8)
    cr.quat[:] = (0, 0, 0, 1)
    cr.developed[:] = 1
    cr.expansion[:] = 1.2
    em = upload(cr, cfg, engine)
    em.set_development(cr.developed, cr.expansion)
    sc = fg.ScanConfig(48, 48, 4, 0, 0.25)
    buf, _ = fg.scan_emulsion(em, sc, 3)
    ref = orc.scan(cr, cfg, sc, 3, want_hits=True)
    assert (np.abs(buf - ref["T64"]) / ref["T64"]).max() <= T_RTOL
    np.testing.assert_array_equal(fg.scan_ray_hits(em, sc, 3), ref["ray_hits"])
    assert engine.timings()["fallbacks"] > 0


def test_empty_single_and_zero_opacity(engine):
    cfg = reference_cfg("tri-x", 8.0, 8.0)
    empty = fg.VirtualEmulsionLayer.from_crystals(cfg, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 4)),
                                                  np.zeros(0), None, engine)
    assert len(empty) == 0
    fg.expose_emulsion(empty, np.ones((4, 4), np.float32), tile_worker_exposure_cfg(), 1)
    rep = fg.develop_emulsion(empty, tile_worker_dev_cfg())
    assert rep.total_crystals == 0
    buf, img = fg.scan_emulsion(empty, fg.ScanConfig(8, 8, 4, 0, 0.25), 1)
    assert (buf == 1.0).all() and (img == 255).all()
    # A unit cube filling pixel (4, 4) exactly: chord 1 for all four strata.
    one = fg.VirtualEmulsionLayer.from_crystals(cfg, [[4.5, 4.5, 7.0]], [[0.5, 0.5, 0.5]], identity_quats(1),
                                                [1.0], None, engine)
    one.set_development([1], [1.0])
    buf, _ = fg.scan_emulsion(one, fg.ScanConfig(8, 8, 4, 0, 0.25), 1)
    assert abs(buf[4, 4] - np.exp(-0.25)) < 1e-6 and buf[0, 0] == 1.0
    buf, _ = fg.scan_emulsion(one, fg.ScanConfig(8, 8, 4, 0, 0.0), 1)
    assert (buf == 1.0).all()


@pytest.mark.parametrize("max_bounces", [0, 1, 2, 5])
def test_production_transport_bounce_limits(engine, max_bounces):
    """The bounce loop's bound (transport.rs:101): the device ends and begins bounces for groups of
    idle lanes and refills lanes whose packets died, so short limits stress those paths.  With no
    bounce nothing is absorbed; with one, two or five the counts follow the oracle's crystal by
    crystal, as at the stock limit (test_c1_production_transport_matches_oracle)."""
    cfg = reference_cfg("tri-x", 96 * C1_PX, 96 * C1_PX)
    cr = orc.synthesize(cfg, 9)
    tile = ramp_tile(96, 96)
    base = tile_worker_exposure_cfg(1.0)
    ecfg = fg.ExposureConfig(base.photons_per_sq_um, base.illumination_angle_rad, base.crystal_absorption_coeff,
                             max_bounces)
    ocr = cr.copy()
    P, _, _ = orc.expose(ocr, cfg, tile, ecfg, 3, orc.FAITHFUL)
    em = upload(cr, cfg, engine)
    fg.expose_emulsion(em, tile, ecfg, 3)
    got = em.latent_counts().astype(np.int64)
    ref = ocr.latent.astype(np.int64)
    assert engine.timings()["photons"] == P
    if max_bounces == 0:
        assert got.sum() == 0 and ref.sum() == 0
        return
    assert ref.sum() > 0
    assert (got == ref).mean() > 0.99
    assert abs(got.sum() - ref.sum()) / ref.sum() < 5e-3


def test_zero_exposure_leaves_no_latent_image(engine):
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    cr = orc.synthesize(cfg, 2)
    em = upload(cr, cfg, engine)
    fg.expose_emulsion(em, np.zeros((8, 8), np.float32), tile_worker_exposure_cfg(), 5)
    assert em.latent_counts().sum() == 0


def test_invalid_arguments_raise(engine):
    cfg = reference_cfg("tri-x", 8.0, 8.0)
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, [[4.0, 4.0, 7.0]], [[0.5, 0.5, 0.5]], identity_quats(1),
                                               [1.0], None, engine)
    with pytest.raises(fg.GpuError) as ei:
        fg.scan_emulsion(em, fg.ScanConfig(0, 8, 4, 0, 0.25), 1)
    assert ei.value.status == 16
    with pytest.raises(fg.GpuError):
        fg.scan_emulsion(em, fg.ScanConfig(8, 8, 1024, 0, 0.25), 1)
