"""GPU tests of the differentiable scan and its hand-written adjoint.

The device forward S = OTF_s(e T) is checked against the FP64 oracle, and the device adjoint
(gradients with respect to per-crystal opacity, exposure multiplier and OTF width) against the
oracle's FP64 adjoint, which tests/test_oracle_adjoint.py pins to central differences.  The loss is
the one of the differentiation configuration: the mean squared difference to a target scanned with
the OTF width scaled by 1.2 and the exposure by 0.9.
"""
import numpy as np
import pytest

import fgrain_gb300 as fg
from oracle import oracle as orc
from tests.helpers import blurred_noise, reference_cfg, tile_worker_dev_cfg, tile_worker_exposure_cfg

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5   # scanned transmittance vs the FP64 oracle
G_RTOL = 1e-4   # gradients vs the FP64 adjoint


def developed_set(preset, w, h, seed, frac=0.5):
    cfg = reference_cfg(preset, w, h)
    cr = orc.synthesize(cfg, seed)
    rng = np.random.default_rng(seed)
    cr.developed[:] = (rng.random(len(cr)) < frac).astype(np.uint8)
    cr.expansion[:] = np.where(cr.developed == 1, 1.2, 0.0)
    sigma = (0.25 + 0.1 * rng.random(len(cr))).astype(np.float32)
    return cfg, cr, sigma


def upload(cfg, cr, engine):
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, cr.pos, cr.dims, cr.quat, cr.sens, cr.morph, engine)
    em.set_development(cr.developed, cr.expansion)
    return em


@pytest.mark.parametrize("preset,size,px,spp", [("t-max", (12.0, 10.0), (24, 20), 4),
                                                 ("tri-x", (20.0, 16.0), (40, 32), 9)])
def test_signal_and_adjoint_match_the_oracle(engine, preset, size, px, spp):
    cfg, cr, sigma = developed_set(preset, *size, 4)
    em = upload(cfg, cr, engine)
    scfg = fg.ScanConfig(px[0], px[1], spp, 0, 0.25)
    s0 = fg.OTF_SIGMA_REFERENCE
    sig64 = sigma.astype(np.float64)
    # Forward.
    S_dev, T_dev = fg.scan_signal(em, scfg, 7, sigma, 1.0, s0)
    S_orc, T_orc = orc.scan_signal(cr, cfg, scfg, 7, sig64, 1.0, s0)
    np.testing.assert_allclose(T_dev, T_orc, rtol=T_RTOL, atol=0)
    np.testing.assert_allclose(S_dev, S_orc, rtol=T_RTOL, atol=0)
    # Target with the OTF width x1.2 and the exposure x0.9, then the MSE gradient at (1, s0).
    tgt, _ = orc.scan_signal(cr, cfg, scfg, 7, sig64, 0.9, 1.2 * s0)
    dL = (2.0 * (S_orc - tgt) / S_orc.size)
    gs_d, ge_d, go_d = fg.scan_backward(em, scfg, 7, dL.astype(np.float32), sigma, 1.0, s0)
    gs_o, ge_o, go_o = orc.scan_backward(cr, cfg, scfg, 7, dL, sig64, 1.0, s0)
    assert abs(ge_d - ge_o) <= G_RTOL * abs(ge_o)
    assert abs(go_d - go_o) <= G_RTOL * abs(go_o)
    assert (gs_d[cr.developed == 0] == 0).all()
    big = np.abs(gs_o) > 1e-3 * np.abs(gs_o).max()
    np.testing.assert_allclose(gs_d[big], gs_o[big], rtol=G_RTOL)
    np.testing.assert_allclose(gs_d, gs_o, rtol=0, atol=G_RTOL * np.abs(gs_o).max())
    em.close()


def test_adjoint_properties_on_a_larger_scan(engine):
    """Size-independent checks on a 256 x 256 t-max scan: linearity in the exposure multiplier and
    the directional derivative along the opacities, both from the device forward."""
    cfg, cr, sigma = developed_set("t-max", 256 / 1.1, 256 / 1.1, 4, frac=0.4)
    em = upload(cfg, cr, engine)
    scfg = fg.ScanConfig(256, 256, 4, 0, 0.25)
    s0 = fg.OTF_SIGMA_REFERENCE
    tgt, _ = fg.scan_signal(em, scfg, 9, sigma, 0.9, 1.2 * s0)
    tgt = tgt.astype(np.float64)

    def loss(sig, e=1.0):
        S, _ = fg.scan_signal(em, scfg, 9, sig, e, s0)
        return np.mean((S.astype(np.float64) - tgt) ** 2), S.astype(np.float64)

    L0, S0 = loss(sigma)
    dL = 2.0 * (S0 - tgt) / S0.size
    gs, ge, go = fg.scan_backward(em, scfg, 9, dL.astype(np.float32), sigma, 1.0, s0)
    # S is linear in e: dL/de = sum dL/dS * S / e exactly.
    assert abs(ge - np.sum(dL * S0)) <= 1e-5 * abs(ge)
    # Directional derivative along sigma (scaling all opacities): central differences of the
    # device forward agree with sum_c sigma_c dL/dsigma_c.
    h = 1e-2
    fd = (loss(sigma * (1 + h))[0] - loss(sigma * (1 - h))[0]) / (2 * h)
    dd = float(np.dot(sigma.astype(np.float64), gs.astype(np.float64)))
    assert abs(dd - fd) <= 2e-3 * abs(fd), (dd, fd)
    assert np.isfinite(go)
    em.close()


def test_emulsion_synthesize_equals_the_tile_synthesis(engine):
    """Device synthesis of a whole emulsion is the tile synthesis of the batched path: same seed and
    box, the same crystals in the same (Morton) order."""
    p = fg.tile_params("t-max", 1 / 1.1, 96, 80, 1.0, 0.0, 1234)
    b = fg.Batch([p], engine, use_graph=False)
    b.set_exposure([np.zeros((80, 96), np.float32)])
    b.run()
    b.wait()
    c = b.tile_crystals(0)
    b.close()
    cfg = fg.EmulsionConfig.preset("t-max", p.film_w, p.film_h)
    em = fg.VirtualEmulsionLayer.synthesize(cfg, 1234, engine)
    d = em.crystals()
    assert len(em) == len(c["pos"]) > 1000
    for k in ("pos", "dims", "quat", "sensitivity", "morphology"):
        np.testing.assert_array_equal(d[k], c[k])
    em.close()


def test_differentiation_configuration_full_size(engine):
    """The differentiation configuration at its full size, checked as it is specified: a 2048 x 2048
    t-max scan (film of 2048 / 1.1 um square, about 24 M crystals) with the developed mask of the
    seed-4 pipeline run (device synthesis with seed 4, exposure of a blurred-noise image at three
    times the tile worker's photons, seed 5, development with the t-max tile-worker settings).
    Loss: MSE to a target scanned with the OTF width x1.2 and the exposure x0.9.  The device
    adjoint's gradients with respect to the exposure multiplier, the OTF width and a sample of
    per-crystal opacities are compared with FP64 central differences (h = 1e-3) of the oracle's FP64
    forward on the device's crystals and mask: the full image for the exposure and the OTF width,
    and for each sampled crystal the pixel window its rays can reach (the tree over all developed
    crystals is the full one, so the window's transmittance is the full image's there)."""
    side_px = 2048
    px = 1.0 / 1.1
    cfg = fg.EmulsionConfig.preset("t-max", side_px * px, side_px * px)
    em = fg.VirtualEmulsionLayer.synthesize(cfg, 4, engine)
    n = len(em)
    assert n > 20_000_000
    exposure = blurred_noise(side_px, side_px, 16.0, 4)
    fg.expose_emulsion(em, exposure, tile_worker_exposure_cfg(3.0), 5)
    fg.develop_emulsion(em, tile_worker_dev_cfg("t-max"))
    dev, _, expn = em.development()
    assert 0.05 < dev.mean() < 0.8
    rng = np.random.default_rng(4)
    sigma = (0.2 + 0.1 * rng.random(n)).astype(np.float32)  # per-crystal silver optical density
    sig64 = sigma.astype(np.float64)
    scfg = fg.ScanConfig(side_px, side_px, 4, 0, 0.25)
    s0, h = fg.OTF_SIGMA_REFERENCE, 1e-3
    # The FP64 forward on the device's own crystals and mask.
    c = em.crystals()
    cr = orc.Crystals(c["pos"], c["dims"], c["quat"], c["sensitivity"], c["morphology"])
    cr.developed[:] = dev
    cr.expansion[:] = expn
    S1, T64 = orc.scan_signal(cr, cfg, scfg, 4, sig64, 1.0, s0)
    tgt = 0.9 * orc.otf_image(T64, 1.2 * s0)
    N = S1.size

    def loss(e, s):
        return np.mean((e * orc.otf_image(T64, s) - tgt) ** 2)

    dL = 2.0 * (S1 - tgt) / N
    gs, ge, go = fg.scan_backward(em, scfg, 4, dL.astype(np.float32), sigma, 1.0, s0)
    assert np.isfinite(gs).all() and (gs[dev == 0] == 0).all()
    fe = (loss(1.0 + h, s0) - loss(1.0 - h, s0)) / (2 * h)
    fo = (loss(1.0, s0 + h) - loss(1.0, s0 - h)) / (2 * h)
    assert abs(ge - fe) <= G_RTOL * abs(fe), (ge, fe)
    assert abs(go - fo) <= G_RTOL * abs(fo), (go, fo)
    # Per-crystal opacities: the four largest gradients and four more drawn among the developed
    # crystals whose gradient is at least 1e-3 of the largest (smaller ones sit at float32's floor).
    mag = np.abs(gs.astype(np.float64))
    top = list(np.argsort(-mag)[:4])
    pool = np.flatnonzero((dev == 1) & (mag >= 1e-3 * mag.max()))
    pick = top + list(rng.choice(np.setdiff1d(pool, top), 4, replace=False))
    wins = []
    for k in pick:
        reach = np.sqrt(3.0) * cr.dims[k].max() * cr.expansion[k] * 1.001
        x0 = max(int(np.floor((cr.pos[k, 0] - reach) / px)) - 1, 0)
        y0 = max(int(np.floor((cr.pos[k, 1] - reach) / px)) - 1, 0)
        x1 = min(int(np.ceil((cr.pos[k, 0] + reach) / px)) + 2, side_px)
        y1 = min(int(np.ceil((cr.pos[k, 1] + reach) / px)) + 2, side_px)
        wins.append((x0, y0, x1 - x0, y1 - y0))
    res = orc.scan_windows(cr, cfg, scfg, 4, sig64, wins, pick, h)
    for k, (x0, y0, w, hh), (tb, tp, tm) in zip(pick, wins, res):
        np.testing.assert_array_equal(tb, T64[y0:y0 + hh, x0:x0 + w])
        Tp, Tm = T64.copy(), T64.copy()
        Tp[y0:y0 + hh, x0:x0 + w] = tp
        Tm[y0:y0 + hh, x0:x0 + w] = tm
        fd = (((orc.otf_image(Tp, s0) - tgt) ** 2 - (orc.otf_image(Tm, s0) - tgt) ** 2).sum() / N) / (2 * h)
        assert abs(gs[k] - fd) <= G_RTOL * abs(fd), (k, gs[k], fd)
    em.close()
