"""The oracle's FP64 adjoint of the differentiable scan against FP64 central differences (CPU).

S = OTF_s(e T): the loss is the mean squared difference to a target scanned with the OTF width
scaled by 1.2 and the exposure by 0.9 (the differentiation configuration, on a small t-max film).
"""
import numpy as np

import fgrain_gb300 as fg
from oracle import oracle as orc
from tests.helpers import reference_cfg

H_FD = 1e-3      # central-difference step
G_RTOL = 1e-4    # adjoint vs finite differences (relative)


def setup(seed=4):
    cfg = reference_cfg("t-max", 12.0, 10.0)
    cr = orc.synthesize(cfg, seed)
    rng = np.random.default_rng(seed)
    cr.developed[:] = (rng.random(len(cr)) < 0.5).astype(np.uint8)
    cr.expansion[:] = np.where(cr.developed == 1, 1.2, 0.0)
    scfg = fg.ScanConfig(24, 20, 4, 0, 0.25)
    sigma = 0.25 + 0.1 * rng.random(len(cr))
    return cfg, cr, scfg, sigma


def test_otf_taps_reproduce_the_reference_scanner():
    k, dk = orc.otf_taps(orc.OTF_SIGMA_REFERENCE)
    np.testing.assert_allclose(k, [0.035, 0.93, 0.035], rtol=1e-12)
    assert abs(sum(dk)) < 1e-12  # the taps stay normalised


def test_adjoint_matches_central_differences():
    cfg, cr, scfg, sigma = setup()
    s0 = orc.OTF_SIGMA_REFERENCE
    tgt, _ = orc.scan_signal(cr, cfg, scfg, 7, sigma, 0.9, 1.2 * s0)

    def loss(sig, e, s):
        S, _ = orc.scan_signal(cr, cfg, scfg, 7, sig, e, s)
        return np.mean((S - tgt) ** 2), S

    e, s = 1.0, s0
    _, S0 = loss(sigma, e, s)
    dL = 2.0 * (S0 - tgt) / S0.size
    gs, ge, go = orc.scan_backward(cr, cfg, scfg, 7, dL, sigma, e, s)
    fe = (loss(sigma, e + H_FD, s)[0] - loss(sigma, e - H_FD, s)[0]) / (2 * H_FD)
    fo = (loss(sigma, e, s + H_FD)[0] - loss(sigma, e, s - H_FD)[0]) / (2 * H_FD)
    assert abs(ge - fe) <= G_RTOL * abs(fe)
    assert abs(go - fo) <= G_RTOL * abs(fo)
    assert (gs[cr.developed == 0] == 0).all()
    for i in np.argsort(-np.abs(gs))[:6]:
        sp, sm = sigma.copy(), sigma.copy()
        sp[i] += H_FD
        sm[i] -= H_FD
        fd = (loss(sp, e, s)[0] - loss(sm, e, s)[0]) / (2 * H_FD)
        assert abs(gs[i] - fd) <= G_RTOL * abs(fd), (i, gs[i], fd)


def test_signal_is_linear_in_exposure_and_matches_the_scan():
    cfg, cr, scfg, sigma = setup(5)
    S1, T = orc.scan_signal(cr, cfg, scfg, 3, sigma, 1.0)
    S2, _ = orc.scan_signal(cr, cfg, scfg, 3, sigma, 2.5)
    np.testing.assert_allclose(S2, 2.5 * S1, rtol=1e-14)
    r = orc.scan(cr, cfg, scfg, 3, sigma_c=sigma)
    np.testing.assert_array_equal(T, r["T64"])
