"""Whole photographs through the device film renderer (image_pipeline.rs:18-113, 299-891,
1017-1085), over the C ABI's fg_render_film and its stage entry points.

``FilmRenderOptions`` mirrors the reference's struct field for field (the ``gpu`` switch has no
meaning here: everything runs on the device).  ``render_film_black_and_white_tiled`` and
``render_film_color_tiled`` take a u8 image (H, W) or (H, W, 3) and return the rendered u8 image
and an ``ImageProcessReport``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi

TRIANGLE = 0
LANCZOS3 = 1


@dataclass
class FilmRenderOptions:
    preset: str = "tri-x"
    grain_size_px: float = 2.2
    grain_strength: float = 1.0
    exposure: float = 1.0
    color: bool = False
    output_resolution: tuple | None = None
    tile_size: int = 320
    seed: int = 42
    gpu: bool = True
    auto_scale: bool = False
    scale: float = 1.0
    reference_res: int = 6000
    supersample: int = 1
    push: float = 0.0
    eberhard: float = 1.0
    scanner_otf: bool = True
    batch_bytes: int = 0  # device bytes one batch of tiles may use (0: 70 % of the free memory)

    def to_c(self) -> _abi.fg_film_options:
        o = _abi.fg_film_options()
        o.preset = self.preset.encode()  # the structure keeps the bytes alive
        o.grain_size_px = self.grain_size_px
        o.grain_strength = self.grain_strength
        o.exposure = self.exposure
        o.color = int(bool(self.color))
        ow, oh = self.output_resolution or (0, 0)
        o.out_w, o.out_h = int(ow), int(oh)
        o.tile_size = int(self.tile_size)
        o.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        o.auto_scale = int(bool(self.auto_scale))
        o.reference_res = int(self.reference_res)
        o.scale = self.scale
        o.supersample = int(self.supersample)
        o.scanner_otf = int(bool(self.scanner_otf))
        o.push = self.push
        o.eberhard = self.eberhard
        o.batch_bytes = int(self.batch_bytes)
        return o


@dataclass
class ImageProcessReport:
    """image_pipeline.rs:97-105, plus the photons launched and the device stage times (``extra``).
    Totals are summed over all tiles of all layers (the reference reports a colour render as its
    red layer's totals times three)."""
    input_resolution: tuple
    output_resolution: tuple
    total_tiles: int
    total_crystals: int
    developed_crystals: int
    total_clumps: int
    elapsed_seconds: float
    photons: int = 0
    extra: dict = field(default_factory=dict)


def _u8(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def _f32(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _engine(engine):
    from .api import _engine as eng

    return eng(engine)


def _run(engine, fn, *args):
    from .api import _check

    e = _engine(engine)
    _check(e, getattr(e._lib, fn)(e._h, *args))


def render_film(image, options: FilmRenderOptions | None = None, engine=None):
    """Renders a u8 image ((H, W) gray or (H, W, 3) RGB) on the device: a gray image (or the
    stock's panchromatic luma of an RGB one), or three dye layers when options.color is set."""
    opts = options or FilmRenderOptions()
    img = np.ascontiguousarray(image, np.uint8)
    if img.ndim not in (2, 3) or (img.ndim == 3 and img.shape[2] != 3):
        raise ValueError("image must be (H, W) or (H, W, 3) u8")
    h, w = img.shape[:2]
    ch = 1 if img.ndim == 2 else 3
    co = opts.to_c()
    lib = _abi.load()
    ow, oh = C.c_uint32(), C.c_uint32()
    if lib.fg_film_output_size(C.byref(co), w, h, C.byref(ow), C.byref(oh)) != 0:
        raise ValueError("bad output size")
    out = np.zeros((oh.value, ow.value, 3) if opts.color else (oh.value, ow.value), np.uint8)
    rep = _abi.fg_film_report()
    _run(engine, "fg_render_film", _u8(img), w, h, ch, C.byref(co), _u8(out), C.byref(rep))
    return ImageProcessReport((rep.in_w, rep.in_h), (rep.out_w, rep.out_h), rep.total_tiles, rep.total_crystals,
                              rep.developed_crystals, rep.total_clumps, rep.elapsed_seconds, rep.photons,
                              {"prep_ms": rep.prep_ms, "tiles_ms": rep.tiles_ms, "finish_ms": rep.finish_ms}), out


def render_film_black_and_white_tiled(image, options: FilmRenderOptions | None = None, engine=None):
    opts = options or FilmRenderOptions()
    opts = FilmRenderOptions(**{**opts.__dict__, "color": False}) if opts.color else opts
    return render_film(image, opts, engine)


def render_film_color_tiled(image, options: FilmRenderOptions | None = None, engine=None):
    img = np.asarray(image, np.uint8)
    if img.ndim == 2:
        img = np.repeat(img[:, :, None], 3, axis=2)
    opts = FilmRenderOptions(**{**(options or FilmRenderOptions()).__dict__, "color": True})
    return render_film(img, opts, engine)


# ---- stages (parity checks and custom pipelines) ----

def panchromatic_luma(rgb, preset: str, engine=None) -> np.ndarray:
    a = np.ascontiguousarray(rgb, np.uint8)
    out = np.zeros(a.shape[:2], np.uint8)
    _run(engine, "fg_panchromatic_luma", _u8(a), a.shape[1], a.shape[0], preset.encode(), _u8(out))
    return out


def resize_u8(img, ow: int, oh: int, filt: int, engine=None) -> np.ndarray:
    a = np.ascontiguousarray(img, np.uint8)
    out = np.zeros((oh, ow), np.uint8)
    _run(engine, "fg_resize_u8", _u8(a), a.shape[1], a.shape[0], ow, oh, filt, _u8(out))
    return out


def gelatin_psf(img, engine=None):
    """(h_effective, gate (top, bottom, left, right)) of a u8 image."""
    a = np.ascontiguousarray(img, np.uint8)
    out = np.zeros(a.shape, np.float32)
    gate = (C.c_uint32 * 4)()
    _run(engine, "fg_gelatin_psf", _u8(a), a.shape[1], a.shape[0], _f32(out), gate)
    return out, tuple(gate)


def film_finish(preset, grain_px, strength, push, scanner_otf, out_w, out_h, grid, step, pad, densities, src, heff,
                fields=False, engine=None):
    """image_pipeline.rs:593-891 on given tile densities: (u8 image, stats[, 5 field planes])."""
    pb = preset.encode()
    cfg = _abi.fg_finish_cfg(pb, grain_px, strength, push, int(bool(scanner_otf)), 0)
    desc = np.array([[t.tx, t.ty, t.x_start, t.y_start, t.tw, t.th] for t in grid], np.uint32).ravel()
    ds = [np.ascontiguousarray(d, np.float32) for d in densities]
    ptrs = (C.POINTER(C.c_float) * len(ds))(*[_f32(d) for d in ds])
    s = np.ascontiguousarray(src, np.uint8)
    he = np.ascontiguousarray(heff, np.float32)
    out = np.zeros((out_h, out_w), np.uint8)
    fl = np.zeros((5, out_h, out_w), np.float32) if fields else None
    st = np.zeros(4, np.float32)
    _run(engine, "fg_film_finish", C.byref(cfg), out_w, out_h, step, pad, len(ds),
         desc.ctypes.data_as(C.POINTER(C.c_uint32)), ptrs, _u8(s), _f32(he), _u8(out),
         _f32(fl) if fields else None, _f32(st))
    return (out, st, fl) if fields else (out, st)
