"""Shared helpers for the tests: configs and synthetic inputs."""
from __future__ import annotations

import numpy as np

import fgrain_gb300 as fg


def identity_quats(n):
    q = np.zeros((n, 4))
    q[:, 3] = 1.0
    return q


def blurred_noise(h, w, sigma, seed, gamma=None):
    """Uniform [0,1) noise from numpy's PCG64 seed, Gaussian-blurred (reflect), optional gamma."""
    from scipy.ndimage import gaussian_filter

    a = np.random.default_rng(seed).random((h, w))
    b = gaussian_filter(a, sigma, mode="reflect")
    if gamma is not None:
        b = np.clip(b, 0.0, None) ** gamma
    return b.astype(np.float32)


def tile_worker_exposure_cfg(exposure=1.0):
    """ExposureConfig of the tile worker (image_pipeline.rs:942-947)."""
    return fg.ExposureConfig(6.0 * max(exposure, 0.05), 0.12, 1.3, 48)


def tile_worker_dev_cfg(preset="tri-x", push=0.0):
    """DevelopmentConfig of the tile worker (image_pipeline.rs:963-976)."""
    if preset == "t-max":
        fe, prox = 1.10 + 0.04 * push, 1.10 + 0.03 * push
    elif preset == "hp5":
        fe, prox = 1.15 + 0.05 * push, 1.18 + 0.04 * push
    else:
        fe, prox = 1.20 + 0.06 * push, 1.25 + 0.05 * push
    return fg.DevelopmentConfig(4, fe, prox, 0.85 + 0.05 * push)


# The four film stocks exactly as emulsion.rs:46-136 defines them (depth, r_min, mean radius,
# size variance, morphology, aspect ratio, optics (n, mu_a, mu_s, g, R_ahu, OD), sensitivity).
REFERENCE_PRESETS = {
    "tri-x": (14.0, 1.2, 0.55, 0.40, 0, 1.0, (1.534, 0.003, 0.050, 0.80, 0.14, 0.80), 1.2),
    "tri-x-1600": (14.5, 1.1, 0.52, 0.38, 0, 1.0, (1.534, 0.0032, 0.052, 0.80, 0.14, 0.80), 1.35),
    "t-max": (8.0, 0.9, 0.40, 0.20, 1, 6.5, (1.534, 0.002, 0.035, 0.85, 0.08, 1.10), 0.8),
    "hp5": (12.5, 1.1, 0.50, 0.30, 2, 1.0, (1.534, 0.0025, 0.045, 0.82, 0.12, 0.85), 1.1),
}


def reference_cfg(name, w, h):
    d, r, m, v, mo, ar, o, s = REFERENCE_PRESETS[name]
    return fg.EmulsionConfig((w, h, d), r, m, v, fg.Morphology(mo), ar, fg.GelatinOptics(*o), s)


def tile_cfg(p):
    """The emulsion configuration a tile's parameters describe (the stock the tile worker selected
    for its push, on the tile's film box)."""
    o = fg.GelatinOptics(*[getattr(p.optics, k) for k, _ in p.optics._fields_])
    return fg.EmulsionConfig((p.film_w, p.film_h, p.film_d), p.r_min, p.mean_crystal_radius, p.size_variance,
                             fg.Morphology(p.morphology), p.tabular_aspect_ratio, o, p.base_sensitivity)
