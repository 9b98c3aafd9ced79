"""Python mirror of fgrain's photon-transport and scan entry points over the C ABI.

Names, argument meaning and defaults follow the reference crate (paths relative to fgrain):
``EmulsionConfig`` (src/emulsion.rs:14-137), ``ExposureConfig`` (src/transport.rs:15-39),
``DevelopmentConfig`` / ``DevelopmentReport`` (src/development.rs:12-56), ``ScanConfig`` /
``ScanMode`` (src/transmittance.rs:17-60), ``expose_emulsion`` (src/transport.rs:48),
``develop_emulsion`` (src/development.rs:59), ``scan_emulsion`` (src/transmittance.rs:65),
``GpuEngine`` / ``get_gpu_engine`` (src/gpu.rs:9-14,155) and ``GpuError`` (src/error.rs:9-33).

Every call runs on the GPU through libfgrain_cuda.so; a failure raises ``GpuError`` carrying
the C status.  The exposure closure of ``expose_emulsion`` cannot cross a C ABI, so it takes
the sampled exposure tile (the tile worker's closure, src/image_pipeline.rs:949-958).
"""
from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _abi


class GpuError(RuntimeError):
    """A non-OK fg_status (codes 1-6 mirror GpuError's variants)."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.name = _abi.STATUS_NAMES.get(status, str(status))
        super().__init__(f"{self.name}: {message}")


class Morphology(IntEnum):
    Cubic = 0
    Tabular = 1
    Octahedral = 2


class ScanMode(IntEnum):
    NegativeTransmittance = 0
    PositivePrint = 1
    OpticalDensity = 2


@dataclass
class GelatinOptics:
    refractive_index: float = 1.534
    absorption_coeff: float = 0.002
    scattering_coeff: float = 0.045
    anisotropy_g: float = 0.82
    antihalation_reflectance: float = 0.12
    antihalation_density: float = 0.85


@dataclass
class EmulsionConfig:
    dimensions: tuple = (100.0, 100.0, 14.0)
    r_min: float = 1.2
    mean_crystal_radius: float = 0.55
    size_variance: float = 0.40
    morphology: Morphology = Morphology.Cubic
    tabular_aspect_ratio: float = 1.0
    optics: GelatinOptics = field(default_factory=GelatinOptics)
    base_sensitivity: float = 1.2

    @classmethod
    def preset(cls, name: str, width: float, height: float) -> "EmulsionConfig":
        c = _abi.fg_emulsion_cfg()
        _check(None, _abi.load().fg_emulsion_preset(name.encode(), width, height, C.byref(c)))
        return cls.from_c(c)

    @classmethod
    def tri_x_400(cls, w, h):
        return cls.preset("tri-x", w, h)

    @classmethod
    def tri_x_1600(cls, w, h):
        return cls.preset("tri-x-1600", w, h)

    @classmethod
    def t_max_100(cls, w, h):
        return cls.preset("t-max", w, h)

    @classmethod
    def hp5_plus(cls, w, h):
        return cls.preset("hp5", w, h)

    @classmethod
    def from_c(cls, c) -> "EmulsionConfig":
        o = c.optics
        return cls((c.width, c.height, c.depth), c.r_min, c.mean_crystal_radius, c.size_variance,
                   Morphology(c.morphology), c.tabular_aspect_ratio,
                   GelatinOptics(o.refractive_index, o.absorption_coeff, o.scattering_coeff,
                                 o.anisotropy_g, o.antihalation_reflectance, o.antihalation_density),
                   c.base_sensitivity)

    def to_c(self) -> _abi.fg_emulsion_cfg:
        o = self.optics
        return _abi.fg_emulsion_cfg(
            float(self.dimensions[0]), float(self.dimensions[1]), float(self.dimensions[2]),
            self.r_min, self.mean_crystal_radius, self.size_variance, int(self.morphology), 0,
            self.tabular_aspect_ratio,
            _abi.fg_optics(o.refractive_index, o.absorption_coeff, o.scattering_coeff,
                           o.anisotropy_g, o.antihalation_reflectance, o.antihalation_density),
            self.base_sensitivity)


@dataclass
class ExposureConfig:
    photons_per_sq_um: float = 50.0
    illumination_angle_rad: float = 0.15
    crystal_absorption_coeff: float = 1.2
    max_bounces: int = 64

    def to_c(self):
        return _abi.fg_exposure_cfg(self.photons_per_sq_um, self.illumination_angle_rad,
                                    self.crystal_absorption_coeff, int(self.max_bounces), 0)


@dataclass
class DevelopmentConfig:
    threshold_photons: int = 3
    filament_expansion: float = 1.8
    clumping_proximity_factor: float = 1.25
    developer_contrast: float = 0.75

    def to_c(self):
        return _abi.fg_dev_cfg(int(self.threshold_photons), 0, self.filament_expansion,
                               self.clumping_proximity_factor, self.developer_contrast)


@dataclass
class DevelopmentReport:
    total_crystals: int = 0
    developed_crystals: int = 0
    fixed_crystals: int = 0
    total_clumps: int = 0
    max_clump_size: int = 0
    avg_clump_size: float = 0.0


@dataclass
class ScanConfig:
    width_px: int = 512
    height_px: int = 512
    samples_per_pixel: int = 16
    mode: ScanMode = ScanMode.PositivePrint
    silver_opacity: float = 25.0

    def to_c(self):
        return _abi.fg_scan_cfg(int(self.width_px), int(self.height_px),
                                int(self.samples_per_pixel), int(self.mode), self.silver_opacity)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def _check(engine, status: int):
    if status != _abi.FG_OK:
        msg = _abi.load().fg_last_error(engine._h).decode() if engine is not None else ""
        raise GpuError(status, msg)


class GpuEngine:
    """One CUDA device and stream; calls are serialised like the reference's dispatch lock."""

    def __init__(self, device: int = 0):
        self._lib = _abi.load()
        h = C.c_void_p()
        st = self._lib.fg_engine_create(device, C.byref(h))
        if st != _abi.FG_OK:
            raise GpuError(st, "engine creation failed")
        self._h = h

    def adapter_name(self) -> str:
        return self._lib.fg_engine_device_name(self._h).decode()

    def timings(self) -> dict:
        t = _abi.fg_timings()
        _check(self, self._lib.fg_engine_timings(self._h, C.byref(t)))
        return {name: getattr(t, name) for name, _ in t._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fg_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ENGINE = None
_ENGINE_ERR = None
_ENGINE_LOCK = threading.Lock()


def get_gpu_engine():
    """Process-wide engine, created on first use; None when no device can be used (gpu.rs:9-14)."""
    global _ENGINE, _ENGINE_ERR
    with _ENGINE_LOCK:
        if _ENGINE is None and _ENGINE_ERR is None:
            try:
                _ENGINE = GpuEngine(0)
            except GpuError as e:
                _ENGINE_ERR = e
        return _ENGINE


def _engine(engine):
    e = engine or get_gpu_engine()
    if e is None:
        raise GpuError(1, str(_ENGINE_ERR) if _ENGINE_ERR else "no CUDA device")
    return e


class VirtualEmulsionLayer:
    """A crystal set resident on the device (VirtualEmulsionLayer, src/emulsion.rs:141-226)."""

    def __init__(self, engine: GpuEngine, config: EmulsionConfig, handle):
        self.engine = engine
        self.config = config
        self._h = handle

    @classmethod
    def synthesize(cls, config: EmulsionConfig, seed: int, engine: GpuEngine | None = None) -> "VirtualEmulsionLayer":
        """VirtualEmulsionLayer::synthesize (emulsion.rs:155-220), on the device."""
        e = _engine(engine)
        cfg = config.to_c()
        h = C.c_void_p()
        _check(e, e._lib.fg_emulsion_synthesize(e._h, C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF, C.byref(h)))
        return cls(e, config, h.value)

    @classmethod
    def from_crystals(cls, config: EmulsionConfig, pos, dims, quat, sensitivity, morphology=None,
                      engine: GpuEngine | None = None) -> "VirtualEmulsionLayer":
        e = _engine(engine)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        dims = np.ascontiguousarray(dims, dtype=np.float64).reshape(n, 3)
        quat = np.ascontiguousarray(quat, dtype=np.float64).reshape(n, 4)
        sens = np.ascontiguousarray(sensitivity, dtype=np.float64).reshape(n)
        morph = None if morphology is None else np.ascontiguousarray(morphology, dtype=np.int32).reshape(n)
        host = _abi.fg_crystals_host(_ptr(pos, C.c_double), _ptr(dims, C.c_double),
                                     _ptr(quat, C.c_double), _ptr(sens, C.c_double),
                                     _ptr(morph, C.c_int32))
        cfg = config.to_c()
        h = C.c_void_p()
        _check(e, e._lib.fg_emulsion_upload(e._h, C.byref(cfg), C.byref(host), n, C.byref(h)))
        return cls(e, config, h)

    def __len__(self) -> int:
        n = C.c_size_t()
        _check(self.engine, self.engine._lib.fg_emulsion_count(self._h, C.byref(n)))
        return n.value

    def crystals(self) -> dict:
        n = len(self)
        out = {"pos": np.zeros((n, 3)), "dims": np.zeros((n, 3)), "quat": np.zeros((n, 4)),
               "sensitivity": np.zeros(n), "morphology": np.zeros(n, np.int32)}
        o = _abi.fg_crystals_out(_ptr(out["pos"], C.c_double), _ptr(out["dims"], C.c_double),
                                 _ptr(out["quat"], C.c_double), _ptr(out["sensitivity"], C.c_double),
                                 _ptr(out["morphology"], C.c_int32))
        e = self.engine
        _check(e, e._lib.fg_emulsion_download(e._h, self._h, C.byref(o)))
        return out

    def latent_counts(self) -> np.ndarray:
        c = np.zeros(len(self), np.uint32)
        e = self.engine
        _check(e, e._lib.fg_emulsion_get_counts(e._h, self._h, _ptr(c, C.c_uint32)))
        return c

    def set_latent_counts(self, counts) -> None:
        c = np.ascontiguousarray(counts, dtype=np.uint32)
        assert c.shape == (len(self),)
        e = self.engine
        _check(e, e._lib.fg_emulsion_set_counts(e._h, self._h, _ptr(c, C.c_uint32)))

    def development(self):
        n = len(self)
        dv = np.zeros(n, np.uint8)
        cl = np.zeros(n, np.int64)
        ex = np.zeros(n, np.float64)
        e = self.engine
        _check(e, e._lib.fg_emulsion_get_development(e._h, self._h, _ptr(dv, C.c_uint8),
                                                     _ptr(cl, C.c_int64), _ptr(ex, C.c_double)))
        return dv, cl, ex

    def set_development(self, developed, expansion) -> None:
        dv = np.ascontiguousarray(developed, dtype=np.uint8)
        ex = np.ascontiguousarray(expansion, dtype=np.float64)
        e = self.engine
        _check(e, e._lib.fg_emulsion_set_development(e._h, self._h, _ptr(dv, C.c_uint8),
                                                     _ptr(ex, C.c_double)))

    def close(self):
        if getattr(self, "_h", None):
            self.engine._lib.fg_emulsion_destroy(self.engine._h, self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def expose_emulsion(emulsion: VirtualEmulsionLayer, exposure_tile, config: ExposureConfig,
                    seed: int) -> None:
    """Monte-Carlo exposure; latent counts accumulate on the emulsion (transport.rs:48-188)."""
    tile = np.ascontiguousarray(exposure_tile, dtype=np.float32)
    th, tw = tile.shape
    cfg = config.to_c()
    e = emulsion.engine
    _check(e, e._lib.fg_expose_emulsion(e._h, emulsion._h, _ptr(tile, C.c_float), tw, th,
                                        C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF))


def develop_emulsion(emulsion: VirtualEmulsionLayer, config: DevelopmentConfig) -> DevelopmentReport:
    """Threshold, filament expansion and clumping (development.rs:59-188)."""
    cfg = config.to_c()
    rep = _abi.fg_dev_report()
    e = emulsion.engine
    _check(e, e._lib.fg_develop_emulsion(e._h, emulsion._h, C.byref(cfg), C.byref(rep)))
    return DevelopmentReport(rep.total_crystals, rep.developed_crystals, rep.fixed_crystals,
                             rep.total_clumps, rep.max_clump_size, rep.avg_clump_size)


def scan_emulsion(emulsion: VirtualEmulsionLayer, config: ScanConfig, seed: int,
                  sigma_per_crystal=None):
    """Scanner transmittance; returns (buffer float32 [h, w], 8-bit image [h, w])."""
    cfg = config.to_c()
    out = np.zeros((config.height_px, config.width_px), np.float32)
    img = np.zeros((config.height_px, config.width_px), np.uint8)
    sig = None if sigma_per_crystal is None else np.ascontiguousarray(sigma_per_crystal, np.float32)
    e = emulsion.engine
    _check(e, e._lib.fg_scan_emulsion(e._h, emulsion._h, C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF,
                                      _ptr(sig, C.c_float), _ptr(out, C.c_float),
                                      _ptr(img, C.c_uint8)))
    return out, img


OTF_SIGMA_REFERENCE = 0.3904441347190481  # OTF width whose taps are the reference's (0.035, 0.93, 0.035)


def scan_signal(emulsion: VirtualEmulsionLayer, config: ScanConfig, seed: int, sigma_per_crystal=None,
                exposure: float = 1.0, otf_sigma: float = OTF_SIGMA_REFERENCE):
    """Differentiable scan: (signal = OTF_s(exposure * T), T), float32 [h, w] each."""
    cfg = config.to_c()
    S = np.zeros((config.height_px, config.width_px), np.float32)
    T = np.zeros_like(S)
    sig = None if sigma_per_crystal is None else np.ascontiguousarray(sigma_per_crystal, np.float32)
    e = emulsion.engine
    _check(e, e._lib.fg_scan_signal(e._h, emulsion._h, C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF,
                                    _ptr(sig, C.c_float), float(exposure), float(otf_sigma),
                                    _ptr(S, C.c_float), _ptr(T, C.c_float)))
    return S, T


def scan_backward(emulsion: VirtualEmulsionLayer, config: ScanConfig, seed: int, dL_dsignal,
                  sigma_per_crystal=None, exposure: float = 1.0, otf_sigma: float = OTF_SIGMA_REFERENCE):
    """Adjoint of scan_signal: (dL/dsigma per crystal [float32], dL/dexposure, dL/dotf_sigma)."""
    cfg = config.to_c()
    g = np.ascontiguousarray(dL_dsignal, np.float32).reshape(config.height_px, config.width_px)
    gs = np.zeros(len(emulsion), np.float32)
    ge = C.c_double()
    go = C.c_double()
    sig = None if sigma_per_crystal is None else np.ascontiguousarray(sigma_per_crystal, np.float32)
    e = emulsion.engine
    _check(e, e._lib.fg_scan_backward(e._h, emulsion._h, C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF,
                                      _ptr(sig, C.c_float), float(exposure), float(otf_sigma), _ptr(g, C.c_float),
                                      _ptr(gs, C.c_float), C.byref(ge), C.byref(go)))
    return gs, ge.value, go.value


SEGMENT_DTYPE = np.dtype([("origin", "<f8", 3), ("dir", "<f8", 3), ("step", "<f8"),
                          ("energy", "<f8"), ("photon", "<u4"), ("bounce", "<u4")])


REPLAY_IDS_PER_SEGMENT = 64  # room for hit ids per segment in replay_segments' output


def replay_segments(emulsion: VirtualEmulsionLayer, config: ExposureConfig, seed: int, segments):
    """Exact replay of recorded photon segments: the reference's tree walk and hit rule
    (bvh.rs:300-347, crystal.rs:140-217) and its per-hit arithmetic (transport.rs:108-138) in FP64.
    Latent counts are added to the emulsion.  Returns (offsets[n+1], hit ids in absorption order)."""
    segs = np.ascontiguousarray(segments, dtype=SEGMENT_DTYPE)
    n = segs.shape[0]
    offsets = np.zeros(n + 1, np.uint32)
    cap = max(n * REPLAY_IDS_PER_SEGMENT, 1)
    ids = np.zeros(cap, np.uint32)
    nh = C.c_size_t()
    e = emulsion.engine
    cfg = config.to_c()
    _check(e, e._lib.fg_replay_segments(e._h, emulsion._h, C.byref(cfg), seed & 0xFFFFFFFFFFFFFFFF,
                                        segs.ctypes.data_as(C.POINTER(_abi.fg_segment)), n,
                                        _ptr(offsets, C.c_uint32), _ptr(ids, C.c_uint32), cap,
                                        C.byref(nh)))
    if nh.value > cap:
        raise ValueError(f"{nh.value} hits exceed the {cap} ids replay_segments keeps")
    return offsets, ids[: nh.value].copy()


def reference_tree(emulsion: VirtualEmulsionLayer, developed_only=False):
    """The device's copy of the reference tree (bvh.rs:157-295) over the crystals, or over the
    developed ones (the scan's tree): (crystal ids in the tree's index order, leaves as rows of
    (first index, count) sorted by first index, leaf boxes as rows of lo xyz, hi xyz)."""
    e = emulsion.engine
    cap = max(len(emulsion), 1)
    order = np.zeros(cap, np.uint32)
    leaves = np.zeros((cap, 2), np.uint32)
    boxes = np.zeros((cap, 6))
    ne, nl = C.c_size_t(), C.c_size_t()
    _check(e, e._lib.fg_emulsion_reference_tree(e._h, emulsion._h, int(developed_only), _ptr(order, C.c_uint32),
                                                _ptr(leaves, C.c_uint32), _ptr(boxes, C.c_double), cap,
                                                C.byref(ne), C.byref(nl)))
    return order[: ne.value].copy(), leaves[: nl.value].copy(), boxes[: nl.value].copy()


def replay_rays(emulsion: VirtualEmulsionLayer, origins, dirs, developed_only=True):
    """Exact hit lists of arbitrary rays; returns (offsets, ids, chord sums)."""
    o = np.ascontiguousarray(origins, np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, np.float64).reshape(-1, 3)
    n = o.shape[0]
    e = emulsion.engine
    offsets = np.zeros(n + 1, np.uint32)
    nh = C.c_size_t()
    _check(e, e._lib.fg_replay_rays(e._h, emulsion._h, _ptr(o, C.c_double), _ptr(d, C.c_double), n,
                                    int(developed_only), _ptr(offsets, C.c_uint32), None, 0,
                                    C.byref(nh), None))
    cap = nh.value
    ids = np.zeros(max(cap, 1), np.uint32)
    chord = np.zeros(n, np.float64)
    _check(e, e._lib.fg_replay_rays(e._h, emulsion._h, _ptr(o, C.c_double), _ptr(d, C.c_double), n,
                                    int(developed_only), _ptr(offsets, C.c_uint32),
                                    _ptr(ids, C.c_uint32), cap, C.byref(nh), _ptr(chord, C.c_double)))
    return offsets, ids[:cap], chord


def scan_ray_hits(emulsion: VirtualEmulsionLayer, config: ScanConfig, seed: int) -> np.ndarray:
    """Per-ray hit counts of the production scan kernel (pixel-major, stratum-minor)."""
    g = int(round(np.sqrt(max(config.samples_per_pixel, 1))))
    a = max(g * g, 1)
    out = np.zeros(config.width_px * config.height_px * a, np.uint16)
    cfg = config.to_c()
    e = emulsion.engine
    _check(e, e._lib.fg_scan_ray_hits(e._h, emulsion._h, C.byref(cfg), seed, _ptr(out, C.c_uint16)))
    return out


# ------------------------------------------------------------------------------------------------
# Tiles and batches (the drop-in for GpuEngine::render_tile_all_gpu, gpu.rs:491-938, with the CPU
# tile worker's physics, image_pipeline.rs:924-1014).

def tile_params(preset: str, pixel_size_um: float, tw: int, th: int, exposure: float = 1.0,
                push: float = 0.0, tile_seed: int = 0) -> _abi.fg_tile_params:
    """The parameters the reference's CPU tile worker uses for one tile."""
    p = _abi.fg_tile_params()
    _check(None, _abi.load().fg_tile_params_preset(preset.encode(), pixel_size_um, tw, th, exposure, push,
                                                   tile_seed & 0xFFFFFFFFFFFFFFFF, C.byref(p)))
    return p


def render_tile(exposure_tile, params: _abi.fg_tile_params, engine: GpuEngine | None = None) -> np.ndarray:
    """Plain per-tile path: exposure tile -> negative density tile (blocking)."""
    e = _engine(engine)
    tile = np.ascontiguousarray(exposure_tile, np.float32)
    assert tile.shape == (params.height_px, params.width_px)
    out = np.zeros_like(tile)
    _check(e, e._lib.fg_render_tile(e._h, _ptr(tile, C.c_float), C.byref(params), _ptr(out, C.c_float)))
    return out


class Batch:
    """Many tiles rendered by one graph-captured sequence of launches."""

    def __init__(self, params, engine: GpuEngine | None = None, use_graph=True, autotune=False,
                 transport_threads=0, transport_blocks=0, scan_bin_px=0, synth_wait_limit=0, wait_probe=False):
        self.engine = _engine(engine)
        self.params = list(params)
        arr = (_abi.fg_tile_params * len(self.params))(*self.params)
        opt = _abi.fg_batch_options(int(use_graph), int(autotune), transport_threads, transport_blocks,
                                    scan_bin_px, synth_wait_limit, int(bool(wait_probe)), 0)
        h = C.c_void_p()
        e = self.engine
        _check(e, e._lib.fg_batch_create(e._h, arr, len(self.params), C.byref(opt), C.byref(h)))
        self._h = h

    def set_exposure(self, tiles):
        tiles = [np.ascontiguousarray(t, np.float32) for t in tiles]
        for t, p in zip(tiles, self.params):
            assert t.shape == (p.height_px, p.width_px)
        ptrs = (C.POINTER(C.c_float) * len(tiles))(*[_ptr(t, C.c_float) for t in tiles])
        e = self.engine
        _check(e, e._lib.fg_batch_set_exposure(self._h, ptrs))
        self._keep = tiles

    def run(self):
        e = self.engine
        _check(e, e._lib.fg_batch_run(self._h))

    def wait(self) -> dict:
        s = _abi.fg_batch_stats()
        e = self.engine
        _check(e, e._lib.fg_batch_wait(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}

    def time(self, steps: int) -> float:
        """Device milliseconds of `steps` back-to-back replays (CUDA events on the engine stream)."""
        ms = C.c_double()
        e = self.engine
        _check(e, e._lib.fg_batch_time(self._h, steps, C.byref(ms)))
        return ms.value

    def density(self):
        outs = [np.zeros((p.height_px, p.width_px), np.float32) for p in self.params]
        ptrs = (C.POINTER(C.c_float) * len(outs))(*[_ptr(o, C.c_float) for o in outs])
        e = self.engine
        _check(e, e._lib.fg_batch_get_density(self._h, ptrs))
        return outs

    def density_into(self, outs):
        """Copies every tile's density into the given float32 arrays (e.g. page-locked ones)."""
        ptrs = (C.POINTER(C.c_float) * len(outs))(*[_ptr(o, C.c_float) for o in outs])
        e = self.engine
        _check(e, e._lib.fg_batch_get_density(self._h, ptrs))

    def tile_crystals(self, tile: int) -> dict:
        e = self.engine
        n = C.c_size_t()
        _check(e, e._lib.fg_batch_tile_crystals(self._h, tile, None, None, None, None, 0, C.byref(n)))
        k = n.value
        out = {"pos": np.zeros((k, 3)), "dims": np.zeros((k, 3)), "quat": np.zeros((k, 4)),
               "sensitivity": np.zeros(k), "morphology": np.zeros(k, np.int32),
               "counts": np.zeros(k, np.uint32), "developed": np.zeros(k, np.uint8), "expansion": np.zeros(k)}
        o = _abi.fg_crystals_out(_ptr(out["pos"], C.c_double), _ptr(out["dims"], C.c_double),
                                 _ptr(out["quat"], C.c_double), _ptr(out["sensitivity"], C.c_double),
                                 _ptr(out["morphology"], C.c_int32))
        _check(e, e._lib.fg_batch_tile_crystals(self._h, tile, C.byref(o), _ptr(out["counts"], C.c_uint32),
                                                _ptr(out["developed"], C.c_uint8),
                                                _ptr(out["expansion"], C.c_double), k, C.byref(n)))
        return out

    def close(self):
        if getattr(self, "_h", None):
            self.engine._lib.fg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """A numpy view of page-locked host memory (fg_host_alloc)."""

    def __init__(self, shape, dtype=np.float32):
        self._lib = _abi.load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        _check(None, self._lib.fg_host_alloc(self.nbytes, C.byref(p)))
        self._p = p
        buf = (C.c_byte * self.nbytes).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if getattr(self, "_p", None):
            self.array = None
            self._lib.fg_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
