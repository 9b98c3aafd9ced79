"""ctypes wrapper of the CPU oracle (oracle/fg_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
module as the checker.  It restates the reference's Rust CPU path; the product never calls it.
Parity status: geometry, BVH and development are pinned to the reference's inline known-answer
tests; the random streams are not pinned (Philox replaces rand 0.8.8's ChaCha12).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

FAITHFUL = 0
CANONICAL = 1
PRESETS = {"tri-x": 0, "tri-x-1600": 1, "t-max": 2, "hp5": 3}


class or_optics(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("refractive_index", "absorption_coeff", "scattering_coeff",
                                          "anisotropy_g", "antihalation_reflectance",
                                          "antihalation_density")]


class or_emulsion_cfg(C.Structure):
    _fields_ = [("width", C.c_double), ("height", C.c_double), ("depth", C.c_double),
                ("r_min", C.c_double), ("mean_crystal_radius", C.c_double),
                ("size_variance", C.c_double), ("morphology", C.c_int32), ("_pad", C.c_int32),
                ("tabular_aspect_ratio", C.c_double), ("optics", or_optics),
                ("base_sensitivity", C.c_double)]


class or_exposure_cfg(C.Structure):
    _fields_ = [("photons_per_sq_um", C.c_double), ("illumination_angle_rad", C.c_double),
                ("crystal_absorption_coeff", C.c_double), ("max_bounces", C.c_uint32),
                ("_pad", C.c_uint32)]


class or_dev_cfg(C.Structure):
    _fields_ = [("threshold_photons", C.c_uint32), ("_pad", C.c_uint32),
                ("filament_expansion", C.c_double), ("clumping_proximity_factor", C.c_double),
                ("developer_contrast", C.c_double)]


class or_dev_report(C.Structure):
    _fields_ = [("total_crystals", C.c_uint64), ("developed_crystals", C.c_uint64),
                ("fixed_crystals", C.c_uint64), ("total_clumps", C.c_uint64),
                ("max_clump_size", C.c_uint64), ("avg_clump_size", C.c_double)]


class or_scan_cfg(C.Structure):
    _fields_ = [("width_px", C.c_uint32), ("height_px", C.c_uint32),
                ("samples_per_pixel", C.c_uint32), ("mode", C.c_int32),
                ("silver_opacity", C.c_double)]


class or_crystals(C.Structure):
    _fields_ = [("n", C.c_size_t), ("pos", C.POINTER(C.c_double)), ("dims", C.POINTER(C.c_double)),
                ("quat", C.POINTER(C.c_double)), ("sens", C.POINTER(C.c_double)),
                ("morph", C.POINTER(C.c_int32)), ("latent", C.POINTER(C.c_uint32)),
                ("developed", C.POINTER(C.c_uint8)), ("clump", C.POINTER(C.c_int64)),
                ("expansion", C.POINTER(C.c_double))]


class or_tile_report(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("crystals", "developed", "clumps", "photons", "hits")]


SEGMENT_DTYPE = np.dtype([("origin", "<f8", 3), ("dir", "<f8", 3), ("step", "<f8"),
                          ("energy", "<f8"), ("photon", "<u4"), ("bounce", "<u4")])

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", HERE / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()  # no-op when up to date
        _lib = C.CDLL(str(LIB))
        _lib.or_free_path.restype = C.c_double
        _lib.or_rays_hits.restype = C.c_int64
    return _lib


def _p(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class Crystals:
    """Mutable crystal set in crystal-index order (HalideCrystal fields as arrays)."""

    def __init__(self, pos, dims, quat, sens, morph):
        n = len(pos)
        self.pos = np.ascontiguousarray(pos, np.float64).reshape(n, 3)
        self.dims = np.ascontiguousarray(dims, np.float64).reshape(n, 3)
        self.quat = np.ascontiguousarray(quat, np.float64).reshape(n, 4)
        self.sens = np.ascontiguousarray(sens, np.float64).reshape(n)
        self.morph = np.ascontiguousarray(morph, np.int32).reshape(n)
        self.latent = np.zeros(n, np.uint32)
        self.developed = np.zeros(n, np.uint8)
        self.clump = np.full(n, -1, np.int64)
        self.expansion = np.ones(n, np.float64)

    def __len__(self):
        return self.pos.shape[0]

    def struct(self) -> or_crystals:
        return or_crystals(len(self), _p(self.pos, C.c_double), _p(self.dims, C.c_double),
                           _p(self.quat, C.c_double), _p(self.sens, C.c_double),
                           _p(self.morph, C.c_int32), _p(self.latent, C.c_uint32),
                           _p(self.developed, C.c_uint8), _p(self.clump, C.c_int64),
                           _p(self.expansion, C.c_double))

    def copy(self) -> "Crystals":
        c = Crystals(self.pos.copy(), self.dims.copy(), self.quat.copy(), self.sens.copy(), self.morph.copy())
        c.latent = self.latent.copy()
        c.developed = self.developed.copy()
        c.clump = self.clump.copy()
        c.expansion = self.expansion.copy()
        return c


def emulsion_cfg(cfg) -> or_emulsion_cfg:
    """From any object with EmulsionConfig's fields (dimensions tuple + the rest)."""
    o = cfg.optics
    return or_emulsion_cfg(float(cfg.dimensions[0]), float(cfg.dimensions[1]), float(cfg.dimensions[2]),
                           cfg.r_min, cfg.mean_crystal_radius, cfg.size_variance, int(cfg.morphology), 0,
                           cfg.tabular_aspect_ratio,
                           or_optics(o.refractive_index, o.absorption_coeff, o.scattering_coeff,
                                     o.anisotropy_g, o.antihalation_reflectance, o.antihalation_density),
                           cfg.base_sensitivity)


def exposure_cfg(c) -> or_exposure_cfg:
    return or_exposure_cfg(c.photons_per_sq_um, c.illumination_angle_rad, c.crystal_absorption_coeff,
                           int(c.max_bounces), 0)


def dev_cfg(c) -> or_dev_cfg:
    return or_dev_cfg(int(c.threshold_photons), 0, c.filament_expansion, c.clumping_proximity_factor,
                      c.developer_contrast)


def scan_cfg(c) -> or_scan_cfg:
    return or_scan_cfg(int(c.width_px), int(c.height_px), int(c.samples_per_pixel), int(c.mode),
                       c.silver_opacity)


def philox(ctr, key):
    out = (C.c_uint32 * 4)()
    lib().or_philox(*[C.c_uint32(v) for v in ctr], *[C.c_uint32(v) for v in key], out)
    return list(out)


def intersect_crystal(pos, dims, quat, morph, expansion, origin, direction):
    a = lambda v: (C.c_double * len(v))(*v)  # noqa: E731
    t0, t1 = C.c_double(), C.c_double()
    hit = lib().or_intersect_crystal(a(pos), a(dims), a(quat), C.c_int32(morph), C.c_double(expansion),
                                     a(origin), a(direction), C.byref(t0), C.byref(t1))
    return (t0.value, t1.value) if hit else None


def ray_hits(cr: Crystals, origin, direction, mode=FAITHFUL):
    L = lib()
    L.or_ray_hits.restype = C.c_int64
    cap = len(cr) + 1
    idx = np.zeros(cap, np.uint32)
    t0 = np.zeros(cap)
    t1 = np.zeros(cap)
    s = cr.struct()
    a = lambda v: (C.c_double * 3)(*v)  # noqa: E731
    n = L.or_ray_hits(C.byref(s), a(origin), a(direction), mode, _p(idx, C.c_uint32),
                      _p(t0, C.c_double), _p(t1, C.c_double), C.c_int64(cap))
    return idx[:n], t0[:n], t1[:n]


def free_path(optics, xi):
    o = or_optics(optics.refractive_index, optics.absorption_coeff, optics.scattering_coeff,
                  optics.anisotropy_g, optics.antihalation_reflectance, optics.antihalation_density)
    return lib().or_free_path(C.byref(o), C.c_double(xi))


def antihalation(optics, energy, direction, u):
    o = or_optics(optics.refractive_index, optics.absorption_coeff, optics.scattering_coeff,
                  optics.anisotropy_g, optics.antihalation_reflectance, optics.antihalation_density)
    E = C.c_double(energy)
    d = (C.c_double * 3)(*direction)
    alive = lib().or_antihalation(C.byref(o), C.byref(E), d, (C.c_double * 4)(*u))
    return bool(alive), E.value, list(d)


def rays_hits(cr: Crystals, origins, dirs, mode=FAITHFUL, developed_only=False):
    """Hit lists of many rays: (offsets, ids, chord sums)."""
    o = np.ascontiguousarray(origins, np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    n = o.shape[0]
    offsets = np.zeros(n + 1, np.uint32)
    chord = np.zeros(n)
    s = cr.struct()
    total = lib().or_rays_hits(C.byref(s), _p(o, C.c_double), _p(d, C.c_double), C.c_int64(n), mode,
                               int(developed_only), _p(offsets, C.c_uint32), None, C.c_int64(0),
                               _p(chord, C.c_double))
    ids = np.zeros(max(total, 1), np.uint32)
    lib().or_rays_hits(C.byref(s), _p(o, C.c_double), _p(d, C.c_double), C.c_int64(n), mode,
                       int(developed_only), _p(offsets, C.c_uint32), _p(ids, C.c_uint32),
                       C.c_int64(total), _p(chord, C.c_double))
    return offsets, ids[:total], chord


def query_radius(cr: Crystals, center, radius):
    L = lib()
    L.or_query_radius.restype = C.c_int64
    out = np.zeros(len(cr) + 1, np.uint32)
    s = cr.struct()
    n = L.or_query_radius(C.byref(s), (C.c_double * 3)(*center), C.c_double(radius),
                          _p(out, C.c_uint32), C.c_int64(len(out)))
    return sorted(out[:n].tolist())


def bvh_stats(cr: Crystals):
    nodes, depth = C.c_int64(), C.c_int64()
    s = cr.struct()
    lib().or_bvh_stats(C.byref(s), C.byref(nodes), C.byref(depth))
    return nodes.value, depth.value


def bvh_export(cr: Crystals, developed_only=False):
    """The reference tree: (final order of crystal indices, leaves as (start, count) rows, leaf boxes
    (lo xyz, hi xyz) rows), leaves in node order."""
    L = lib()
    L.or_bvh_export.restype = C.c_int64
    n = len(cr)
    order = np.zeros(max(n, 1), np.uint32)
    ls = np.zeros(max(n, 1), np.uint32)
    lc = np.zeros(max(n, 1), np.uint32)
    lb = np.zeros((max(n, 1), 6))
    nl = C.c_int64()
    s = cr.struct()
    m = L.or_bvh_export(C.byref(s), int(developed_only), _p(order, C.c_uint32), C.c_int64(n), _p(ls, C.c_uint32),
                        _p(lc, C.c_uint32), _p(lb, C.c_double), C.c_int64(n), C.byref(nl))
    k = nl.value
    return order[:m].copy(), np.column_stack([ls[:k], lc[:k]]), lb[:k].copy()


def sample_poisson(bounds, r_min, k, seed):
    L = lib()
    L.or_sample_poisson.restype = C.c_int64
    vol = bounds[0] * bounds[1] * bounds[2]
    cap = int(vol / r_min ** 3 * 1.5) + 64
    pts = np.zeros((cap, 3))
    n = L.or_sample_poisson((C.c_double * 3)(*bounds), C.c_double(r_min), C.c_uint32(k),
                            C.c_uint64(seed), _p(pts, C.c_double), C.c_int64(cap))
    assert n <= cap
    return pts[:n].copy()


def synthesize(cfg, seed) -> Crystals:
    L = lib()
    L.or_synthesize.restype = C.c_int64
    ec = emulsion_cfg(cfg)
    vol = ec.width * ec.height * ec.depth
    cap = int(vol / ec.r_min ** 3 * 1.5) + 64
    while True:
        cr = Crystals(np.zeros((cap, 3)), np.zeros((cap, 3)), np.zeros((cap, 4)), np.zeros(cap),
                      np.zeros(cap, np.int32))
        s = cr.struct()
        n = L.or_synthesize(C.byref(ec), C.c_uint64(seed), C.byref(s))
        if n <= cap:
            break
        cap = n
    out = Crystals(cr.pos[:n], cr.dims[:n], cr.quat[:n], cr.sens[:n], cr.morph[:n])
    return out


def expose(cr: Crystals, cfg, tile, ecfg, seed, mode=FAITHFUL, threads=0, record=False):
    """Adds counts into cr.latent; returns (photons, segments or None, absorbing hits)."""
    L = lib()
    L.or_expose.restype = C.c_int64
    tile = np.ascontiguousarray(tile, np.float32)
    th, tw = tile.shape
    ec, xc = emulsion_cfg(cfg), exposure_cfg(ecfg)
    s = cr.struct()
    nseg = C.c_int64()
    hits = C.c_uint64()
    if not record:
        P = L.or_expose(C.byref(s), C.byref(ec), _p(tile, C.c_float), tw, th, C.byref(xc),
                        C.c_uint64(seed), mode, threads, None, C.c_int64(0), None, C.byref(hits))
        return P, None, hits.value
    # Record: first pass sizes the buffer on a copy of the counts.
    saved = cr.latent.copy()
    L.or_expose(C.byref(s), C.byref(ec), _p(tile, C.c_float), tw, th, C.byref(xc), C.c_uint64(seed),
                mode, threads, None, C.c_int64(0), C.byref(nseg), C.byref(hits))
    cr.latent[:] = saved
    segs = np.zeros(nseg.value, SEGMENT_DTYPE)
    s = cr.struct()
    P = L.or_expose(C.byref(s), C.byref(ec), _p(tile, C.c_float), tw, th, C.byref(xc), C.c_uint64(seed),
                    mode, threads, segs.ctypes.data_as(C.c_void_p), C.c_int64(len(segs)),
                    C.byref(nseg), C.byref(hits))
    return P, segs, hits.value


def replay_segments(cr: Crystals, ecfg, seed, segs, mode=FAITHFUL):
    """Replays recorded segments under hit rule `mode`; returns CSR (offsets, crystal ids) in
    absorption order and adds the latent counts to cr.latent."""
    L = lib()
    L.or_replay_segments.restype = C.c_int64
    segs = np.ascontiguousarray(segs, SEGMENT_DTYPE)
    offsets = np.zeros(len(segs) + 1, np.uint32)
    xc = exposure_cfg(ecfg)
    s = cr.struct()
    saved = cr.latent.copy()
    n = L.or_replay_segments(C.byref(s), C.byref(xc), C.c_uint64(seed), segs.ctypes.data_as(C.c_void_p),
                             C.c_int64(len(segs)), mode, _p(offsets, C.c_uint32), None, C.c_int64(0))
    cr.latent[:] = saved
    ids = np.zeros(max(n, 1), np.uint32)
    s = cr.struct()
    L.or_replay_segments(C.byref(s), C.byref(xc), C.c_uint64(seed), segs.ctypes.data_as(C.c_void_p),
                         C.c_int64(len(segs)), mode, _p(offsets, C.c_uint32), _p(ids, C.c_uint32), C.c_int64(n))
    return offsets, ids[:n].copy()


def hit_rule_difference(cr: Crystals, cfg, tile, ecfg, seed, threads=0):
    """How far the canonical hit rule is from the reference's own (FAITHFUL) on one exposure.

    The photon segments of a faithful exposure are replayed under both rules.  Returns the share of
    segments whose hit sets differ, the share of segments whose absorption order differs (same set),
    the relative difference of the total hit count, and, from two full exposures with the same seed,
    the share of crystals whose latent counts differ and the relative difference of the total
    latent photons."""
    c0 = cr.copy()
    c0.latent[:] = 0
    _, segs, _ = expose(c0, cfg, tile, ecfg, seed, FAITHFUL, threads, record=True)
    fa, ca = c0.copy(), c0.copy()
    fa.latent[:] = 0
    ca.latent[:] = 0
    of, idf = replay_segments(fa, ecfg, seed, segs, FAITHFUL)
    oc, idc = replay_segments(ca, ecfg, seed, segs, CANONICAL)
    nseg = len(segs)
    set_diff = order_diff = not_subset = 0
    for k in range(nseg):
        a = idf[of[k]:of[k + 1]]
        b = idc[oc[k]:oc[k + 1]]
        if len(a) != len(b) or not np.array_equal(np.sort(a), np.sort(b)):
            set_diff += 1
            if not np.isin(b, a).all():
                not_subset += 1
        elif not np.array_equal(a, b):
            order_diff += 1
    e_f, e_c = cr.copy(), cr.copy()
    e_f.latent[:] = 0
    e_c.latent[:] = 0
    expose(e_f, cfg, tile, ecfg, seed, FAITHFUL, threads)
    expose(e_c, cfg, tile, ecfg, seed, CANONICAL, threads)
    touched = (e_f.latent > 0) | (e_c.latent > 0)
    return {
        "segments": nseg,
        "segments_hit_set_differs": set_diff / max(nseg, 1),
        "segments_order_differs": order_diff / max(nseg, 1),
        "segments_canonical_not_subset": not_subset,
        "hits_faithful": int(len(idf)), "hits_canonical": int(len(idc)),
        "hits_rel_diff": (len(idf) - len(idc)) / max(len(idc), 1),
        "crystals": len(cr),
        "crystals_count_differs": float((e_f.latent != e_c.latent).mean()),
        "touched_crystals_count_differs": float((e_f.latent != e_c.latent)[touched].mean()) if touched.any() else 0.0,
        "latent_rel_diff": float(e_f.latent.sum(dtype=np.int64) - e_c.latent.sum(dtype=np.int64))
        / max(float(e_c.latent.sum(dtype=np.int64)), 1.0),
    }


def develop(cr: Crystals, dcfg):
    rep = or_dev_report()
    dc = dev_cfg(dcfg)
    s = cr.struct()
    lib().or_develop(C.byref(s), C.byref(dc), C.byref(rep))
    return {k: getattr(rep, k) for k, _ in rep._fields_}


def scan(cr: Crystals, cfg, scfg, seed, mode=FAITHFUL, threads=0, sigma_c=None, want_hits=False):
    """Returns dict(out, image8, T64[, ray_hits])."""
    sc = scan_cfg(scfg)
    ec = emulsion_cfg(cfg)
    h, w = sc.height_px, sc.width_px
    g = int(round(np.sqrt(max(sc.samples_per_pixel, 1))))
    a = max(g * g, 1)
    out = np.zeros((h, w), np.float32)
    img = np.zeros((h, w), np.uint8)
    T64 = np.zeros((h, w), np.float64)
    rh = np.zeros(h * w * a, np.uint16) if want_hits else None
    sig = None if sigma_c is None else np.ascontiguousarray(sigma_c, np.float64)
    s = cr.struct()
    lib().or_scan(C.byref(s), C.byref(ec), C.byref(sc), C.c_uint64(seed), mode, threads,
                  _p(sig, C.c_double), _p(out, C.c_float), _p(img, C.c_uint8), _p(T64, C.c_double),
                  _p(rh, C.c_uint16))
    r = {"out": out, "image8": img, "T64": T64}
    if want_hits:
        r["ray_hits"] = rh
    return r


OTF_SIGMA_REFERENCE = 0.3904441347190481  # otf_taps(s) = (0.035, 0.93, 0.035), the reference's scanner taps


def otf_taps(s):
    k = (C.c_double * 3)()
    dk = (C.c_double * 3)()
    lib().or_otf_taps(C.c_double(s), k, dk)
    return list(k), list(dk)


def scan_signal(cr: Crystals, cfg, scfg, seed, sigma_c=None, exposure=1.0, otf_sigma=OTF_SIGMA_REFERENCE,
                mode=FAITHFUL, threads=0):
    """Differentiable scan S = OTF_s(e T) in FP64; returns (S, T)."""
    sc = scan_cfg(scfg)
    ec = emulsion_cfg(cfg)
    S = np.zeros((sc.height_px, sc.width_px))
    T = np.zeros_like(S)
    sig = None if sigma_c is None else np.ascontiguousarray(sigma_c, np.float64)
    s = cr.struct()
    lib().or_scan_signal(C.byref(s), C.byref(ec), C.byref(sc), C.c_uint64(seed), mode, threads, _p(sig, C.c_double),
                         C.c_double(exposure), C.c_double(otf_sigma), _p(S, C.c_double), _p(T, C.c_double))
    return S, T


def scan_backward(cr: Crystals, cfg, scfg, seed, dL_dS, sigma_c=None, exposure=1.0,
                  otf_sigma=OTF_SIGMA_REFERENCE, mode=FAITHFUL, threads=0):
    """FP64 adjoint of scan_signal: (dL/dsigma per crystal, dL/dexposure, dL/dotf_sigma)."""
    sc = scan_cfg(scfg)
    ec = emulsion_cfg(cfg)
    g = np.ascontiguousarray(dL_dS, np.float64).reshape(sc.height_px, sc.width_px)
    gs = np.zeros(len(cr))
    ge = C.c_double()
    go = C.c_double()
    sig = None if sigma_c is None else np.ascontiguousarray(sigma_c, np.float64)
    s = cr.struct()
    lib().or_scan_backward(C.byref(s), C.byref(ec), C.byref(sc), C.c_uint64(seed), mode, threads,
                           _p(sig, C.c_double), C.c_double(exposure), C.c_double(otf_sigma), _p(g, C.c_double),
                           _p(gs, C.c_double), C.byref(ge), C.byref(go))
    return gs, ge.value, go.value


def scan_windows(cr: Crystals, cfg, scfg, seed, sigma_c, windows, pidx, hstep, threads=0):
    """FP64 transmittance of pixel windows (x0, y0, w, h) under +-hstep on crystal pidx[k]'s opacity,
    with the reference's rule and the tree over all developed crystals: a list of (base, plus,
    minus) arrays of shape (h, w)."""
    L = lib()
    L.or_scan_windows.restype = C.c_int64
    win = np.ascontiguousarray(np.array(windows, np.uint32).reshape(-1, 4))
    pid = np.ascontiguousarray(np.array(pidx, np.uint32).reshape(-1))
    total = int(sum(3 * int(w) * int(h) for _, _, w, h in win))
    out = np.zeros(max(total, 1))
    sig = None if sigma_c is None else np.ascontiguousarray(sigma_c, np.float64)
    s = cr.struct()
    L.or_scan_windows(C.byref(s), C.byref(emulsion_cfg(cfg)), C.byref(scan_cfg(scfg)), C.c_uint64(seed), threads,
                      _p(sig, C.c_double), C.c_int64(len(win)), _p(win, C.c_uint32), _p(pid, C.c_uint32),
                      C.c_double(hstep), _p(out, C.c_double))
    res, base = [], 0
    for _, _, w, h in win:
        n = int(w) * int(h)
        res.append(tuple(out[base + j * n: base + (j + 1) * n].reshape(int(h), int(w)) for j in range(3)))
        base += 3 * n
    return res


def otf_image(field, s):
    """The differentiable scan's OTF in FP64 (or_scan_signal's order: x pass, then y pass), taps of
    otf_taps(s), clamp-to-edge."""
    k, _ = otf_taps(s)
    f = np.asarray(field, np.float64)
    xm = np.concatenate([f[:, :1], f[:, :-1]], axis=1)
    xp = np.concatenate([f[:, 1:], f[:, -1:]], axis=1)
    t = xm * k[0] + f * k[1] + xp * k[2]
    ym = np.concatenate([t[:1], t[:-1]], axis=0)
    yp = np.concatenate([t[1:], t[-1:]], axis=0)
    return ym * k[0] + t * k[1] + yp * k[2]


def scan_ray_origins(cfg, scfg, seed):
    sc = scan_cfg(scfg)
    ec = emulsion_cfg(cfg)
    g = int(round(np.sqrt(max(sc.samples_per_pixel, 1))))
    a = max(g * g, 1)
    o = np.zeros((sc.width_px * sc.height_px * a, 3))
    lib().or_scan_ray_origins(C.byref(ec), C.byref(sc), C.c_uint64(seed), _p(o, C.c_double))
    return o


def render_tile(preset, pixel_size_um, tile, exposure, push, tile_seed, mode=FAITHFUL, threads=0):
    tile = np.ascontiguousarray(tile, np.float32)
    th, tw = tile.shape
    d = np.zeros((th, tw), np.float32)
    rep = or_tile_report()
    lib().or_render_tile(PRESETS[preset] if isinstance(preset, str) else int(preset),
                         C.c_double(pixel_size_um), _p(tile, C.c_float), tw, th, C.c_double(exposure),
                         C.c_double(push), C.c_uint64(tile_seed), mode, threads, _p(d, C.c_float),
                         C.byref(rep))
    return d, {k: getattr(rep, k) for k, _ in rep._fields_}


def scanner_otf(field, taps=(0.035, 0.93, 0.035)):
    f = np.ascontiguousarray(field, np.float32)
    h, w = f.shape
    out = np.zeros_like(f)
    lib().or_scanner_otf(_p(f, C.c_float), w, h, (C.c_float * 3)(*taps), _p(out, C.c_float))
    return out


def blend_tiles(out_w, out_h, grid, step, pad, densities):
    desc = np.array([[t.tx, t.ty, t.x_start, t.y_start, t.tw, t.th] for t in grid], np.uint32).ravel()
    ds = [np.ascontiguousarray(d, np.float32) for d in densities]
    ptrs = (C.POINTER(C.c_float) * len(ds))(*[_p(d, C.c_float) for d in ds])
    out = np.zeros((out_h, out_w), np.float32)
    lib().or_blend_tiles(out_w, out_h, step, pad, len(ds), _p(desc, C.c_uint32), ptrs, _p(out, C.c_float))
    return out


def resize_triangle(field, ow, oh):
    f = np.ascontiguousarray(field, np.float32)
    h, w = f.shape
    out = np.zeros((oh, ow), np.float32)
    lib().or_resize_triangle(_p(f, C.c_float), w, h, ow, oh, _p(out, C.c_float))
    return out


# ---- image stages either side of the tile path (fg_oracle_film.cpp) ----

class or_finish_cfg(C.Structure):
    _fields_ = [("grain_size_px", C.c_double), ("strength", C.c_double), ("push", C.c_double),
                ("base_nominal", C.c_float), ("scanner_otf", C.c_int32)]


def luma_weights(preset):
    w = (C.c_float * 3)()
    lib().or_luma_weights(preset.encode(), w)
    return np.array(list(w), np.float32)


def luma(rgb, preset):
    """Panchromatic luma of an RGB8 image (H, W, 3), image_pipeline.rs:259-296."""
    a = np.ascontiguousarray(rgb, np.uint8)
    h, w = a.shape[:2]
    out = np.zeros((h, w), np.uint8)
    lib().or_luma(_p(a, C.c_uint8), w, h, _p(luma_weights(preset), C.c_float), _p(out, C.c_uint8))
    return out


TRIANGLE, LANCZOS3 = 0, 1


def resize_u8(img, ow, oh, filt):
    a = np.ascontiguousarray(img, np.uint8)
    h, w = a.shape
    out = np.zeros((oh, ow), np.uint8)
    lib().or_resize_u8(_p(a, C.c_uint8), w, h, ow, oh, filt, _p(out, C.c_uint8))
    return out


def gelatin_psf(img):
    """h_effective of a u8 image and its camera gate (top, bottom, left, right)."""
    a = np.ascontiguousarray(img, np.uint8)
    h, w = a.shape
    out = np.zeros((h, w), np.float32)
    gate = (C.c_uint32 * 4)()
    lib().or_gelatin_psf(_p(a, C.c_uint8), w, h, _p(out, C.c_float), gate)
    return out, tuple(gate)


def film_base_nominal(preset):
    L = lib()
    L.or_film_base_nominal.restype = C.c_float
    return float(L.or_film_base_nominal(preset.encode()))


def film_finish(preset, grain_px, strength, push, scanner_otf, out_w, out_h, grid, step, pad, densities, src, heff,
                fields=False):
    """image_pipeline.rs:593-891 on given tile densities: returns (u8 image, stats[, fields])."""
    cfg = or_finish_cfg(grain_px, strength, push, film_base_nominal(preset), int(bool(scanner_otf)))
    desc = np.array([[t.tx, t.ty, t.x_start, t.y_start, t.tw, t.th] for t in grid], np.uint32).ravel()
    ds = [np.ascontiguousarray(d, np.float32) for d in densities]
    ptrs = (C.POINTER(C.c_float) * len(ds))(*[_p(d, C.c_float) for d in ds])
    s = np.ascontiguousarray(src, np.uint8)
    he = np.ascontiguousarray(heff, np.float32)
    out = np.zeros((out_h, out_w), np.uint8)
    fl = np.zeros((5, out_h, out_w), np.float32) if fields else None
    st = np.zeros(4, np.float32)
    lib().or_film_finish(C.byref(cfg), out_w, out_h, step, pad, len(ds), _p(desc, C.c_uint32), ptrs,
                         _p(s, C.c_uint8), _p(he, C.c_float), _p(out, C.c_uint8),
                         _p(fl, C.c_float) if fields else None, _p(st, C.c_float))
    return (out, st, fl) if fields else (out, st)


class FilmTile:
    """One overlapping tile of the image (image_pipeline.rs:400-424)."""

    def __init__(self, idx, tx, ty, x_start, y_start, tw, th):
        self.idx, self.tx, self.ty, self.x_start, self.y_start, self.tw, self.th = idx, tx, ty, x_start, y_start, tw, th


def film_grid(out_w, out_h, grain_px, tile_size):
    """Tile step, pad and tiles (image_pipeline.rs:377-424)."""
    step = max(min(int(np.floor(384.0 * grain_px + 0.5)), tile_size), 48)
    pad = min(max(step // 10, 12), 48)
    ntx, nty = -(-out_w // step), -(-out_h // step)
    tiles = []
    for ty in range(nty):
        for tx in range(ntx):
            x0, y0 = tx * step, ty * step
            xs, ys = max(x0 - pad, 0), max(y0 - pad, 0)
            tiles.append(FilmTile(len(tiles), tx, ty, xs, ys, min(x0 + step + pad, out_w) - xs,
                                  min(y0 + step + pad, out_h) - ys))
    return tiles, step, pad


def film_tile_seed(seed, t):
    """Seed of tile t (image_pipeline.rs:430-434), wrapping at 64 bits."""
    return (seed + t.idx * 73856093 + t.tx * 19349663 + t.ty * 83492791) & 0xFFFFFFFFFFFFFFFF


def film_scaling(opts, out_w, out_h):
    """(grain_size_px, effective_strength, effective_push) of image_pipeline.rs:347-375."""
    user = opts["scale"] if opts["scale"] > 0 else 1.0
    if opts["auto_scale"]:
        ref = max(float(opts["reference_res"]), 512.0)
        ratio = min(max(max(max(out_w, out_h), 1) / ref, 0.05), 5.0)
        res, selwyn = ratio, float(np.sqrt(ratio))
    else:
        res, selwyn = 1.0, 1.0
    grain = min(max(opts["grain_size_px"] * user * res, 0.05), 15.0)
    strength = max(opts["grain_strength"] * float(np.sqrt(user)) * selwyn, 0.0)
    p = opts["preset"].lower()
    push = max(opts["push"], 2.0) if ("1600" in p or p == "caffenol") else max(opts["push"], 0.0)
    return grain, strength, push


FILM_DEFAULTS = dict(preset="tri-x", grain_size_px=2.2, grain_strength=1.0, exposure=1.0, output_resolution=None,
                     tile_size=320, seed=42, auto_scale=False, scale=1.0, reference_res=6000, supersample=1, push=0.0,
                     eberhard=1.0, scanner_otf=True)


def _oracle_stock(preset, push):
    p = preset.lower()
    if p in ("t-max", "tmax"):
        return 2
    if p in ("hp5", "hp5-plus"):
        return 3
    if "1600" in p or p == "caffenol":
        return 1
    return 0


def film_render_bw(image, threads=0, tile_fn=None, **kw):
    """render_film_black_and_white_tiled (image_pipeline.rs:299-891) on the CPU: a u8 gray image
    (H, W) or an RGB8 image (H, W, 3) to a u8 gray image, every tile through or_render_tile, or
    through tile_fn(preset, grain_px, exposure, push, [(tile seed, exposure tile), ...]) -> densities
    when given (a parity check can render the tiles elsewhere and keep this driver)."""
    opts = dict(FILM_DEFAULTS, **kw)
    img = np.ascontiguousarray(image, np.uint8)
    gray = img if img.ndim == 2 else luma(img, opts["preset"])
    in_h, in_w = gray.shape
    aspect = in_w / in_h
    res = opts["output_resolution"]
    if res is None:
        out_w, out_h = in_w, in_h
    elif res[1] == 0:
        out_w, out_h = res[0], max(int(np.floor(res[0] / aspect + 0.5)), 1)
    elif res[0] == 0:
        out_w, out_h = max(int(np.floor(res[1] * aspect + 0.5)), 1), res[1]
    else:
        out_w, out_h = res
    ss = min(max(opts["supersample"], 1), 4)
    if ss > 1:
        big = film_render_bw(image, threads, tile_fn,
                             **dict(opts, supersample=1, output_resolution=(out_w * ss, out_h * ss)))
        return resize_u8(big, out_w, out_h, TRIANGLE)
    src = gray if (in_w, in_h) == (out_w, out_h) else resize_u8(gray, out_w, out_h, LANCZOS3)
    heff, _ = gelatin_psf(src)
    grain, strength, push = film_scaling(opts, out_w, out_h)
    grid, step, pad = film_grid(out_w, out_h, grain, opts["tile_size"])
    stock = _oracle_stock(opts["preset"], push)
    jobs = [(film_tile_seed(opts["seed"], t),
             np.ascontiguousarray(heff[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw])) for t in grid]
    if tile_fn is not None:
        dens = tile_fn(opts["preset"], grain, opts["exposure"], opts["push"], jobs)
    else:
        dens = [render_tile(stock, 1.0 / grain, tile, opts["exposure"], opts["push"], seed, FAITHFUL, threads)[0]
                for seed, tile in jobs]
    out, _ = film_finish(opts["preset"], grain, strength, push, opts["scanner_otf"], out_w, out_h, grid, step, pad,
                         dens, src, heff)
    return out


COLOR_SEED_OFFSETS = (0, 10007, 20011)


def film_render_color(rgb, threads=0, tile_fn=None, **kw):
    """render_film_color_tiled (image_pipeline.rs:1017-1085): the R, G and B channels as three
    black-and-white runs with seeds seed, seed + 10007, seed + 20011 (wrapping), interleaved."""
    opts = dict(FILM_DEFAULTS, **kw)
    img = np.ascontiguousarray(rgb, np.uint8)
    layers = []
    for c, off in enumerate(COLOR_SEED_OFFSETS):
        o = dict(opts, seed=(opts["seed"] + off) & 0xFFFFFFFFFFFFFFFF)
        layers.append(film_render_bw(np.ascontiguousarray(img[..., c]), threads, tile_fn, **o))
    return np.stack(layers, -1)


# ---- the reference's wgpu tile model (fg_oracle_fast.cpp) ----

class or_fast_params(C.Structure):
    _fields_ = [("film_w", C.c_double), ("film_h", C.c_double), ("film_d", C.c_double),
                ("width_px", C.c_uint32), ("height_px", C.c_uint32), ("samples_per_pixel", C.c_uint32),
                ("_pad0", C.c_uint32), ("silver_opacity", C.c_double), ("seed", C.c_uint64),
                ("r_min", C.c_double), ("mean_crystal_radius", C.c_double), ("size_variance", C.c_double),
                ("morphology", C.c_uint32), ("threshold_photons", C.c_uint32),
                ("tabular_aspect_ratio", C.c_double), ("base_sensitivity", C.c_double), ("exposure", C.c_double),
                ("filament_expansion", C.c_double), ("clumping_proximity_factor", C.c_double)]


class or_fast_grid_t(C.Structure):
    _fields_ = [("w", C.c_uint32), ("h", C.c_uint32), ("d", C.c_uint32), ("cell_size", C.c_float)]


FAST_CELL_DTYPE = np.dtype([("pos", "<f4", 4), ("dims_exp", "<f4", 4), ("rot", "<f4", 4), ("flags", "<u4", 4)])


def fast_params(p):
    """or_fast_params from any object with GpuTileParams' field names."""
    q = or_fast_params()
    for name, _ in or_fast_params._fields_:
        if not name.startswith("_"):
            setattr(q, name, getattr(p, name))
    return q


def fast_grid(p):
    g = or_fast_grid_t()
    lib().or_fast_grid(C.byref(fast_params(p)), C.byref(g))
    return (g.w, g.h, g.d), g.cell_size


def fast_tile(p, tile):
    """render_tile_all_gpu's shaders on the CPU: (d_neg, cells as a (d, h, w) record array)."""
    q = fast_params(p)
    t = np.ascontiguousarray(tile, np.float32)
    (w, h, d), _ = fast_grid(p)
    out = np.zeros((q.height_px, q.width_px), np.float32)
    cells = np.zeros((d, h, w), FAST_CELL_DTYPE)
    lib().or_fast_tile(C.byref(q), _p(t, C.c_float), _p(out, C.c_float), C.c_void_p(cells.ctypes.data))
    return out, cells
