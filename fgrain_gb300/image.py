"""Image-level stages of the reference's black-and-white renderer around the tile path.

``tile_grid`` restates image_pipeline.rs:377-424 (tile step from the grain size, overlap pad,
overlapping tile rectangles) and ``tile_seed`` restates image_pipeline.rs:430-434: integer
bookkeeping on the host.  ``blend_tiles`` (image_pipeline.rs:593-649), ``scanner_otf``
(image_pipeline.rs:825-855) and ``resize_triangle`` (the supersample downsample,
image_pipeline.rs:315-330) run on the device through the C ABI.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi

M64 = 0xFFFFFFFFFFFFFFFF


@dataclass(frozen=True)
class Tile:
    idx: int
    tx: int
    ty: int
    x_start: int
    y_start: int
    tw: int
    th: int


def tile_layout(grain_size_px: float, tile_size: int = 320) -> tuple[int, int]:
    """(tile_step, pad): step = clamp(round(384 grain), 48, tile_size), pad = clamp(step/10, 12, 48)."""
    step = max(min(int(np.floor(384.0 * grain_size_px + 0.5)), tile_size), 48)
    step = max(step, 48)
    pad = min(max(step // 10, 12), 48)
    return step, pad


def tile_grid(out_w: int, out_h: int, grain_size_px: float, tile_size: int = 320) -> tuple[list[Tile], int, int]:
    step, pad = tile_layout(grain_size_px, tile_size)
    ntx = (out_w + step - 1) // step
    nty = (out_h + step - 1) // step
    tiles = []
    for ty in range(nty):
        for tx in range(ntx):
            x0, y0 = tx * step, ty * step
            xs, ys = max(x0 - pad, 0), max(y0 - pad, 0)
            xe, ye = min(x0 + step + pad, out_w), min(y0 + step + pad, out_h)
            tiles.append(Tile(len(tiles), tx, ty, xs, ys, xe - xs, ye - ys))
    return tiles, step, pad


def tile_seed(seed: int, t: Tile) -> int:
    return (seed + t.idx * 73856093 + t.tx * 19349663 + t.ty * 83492791) & M64


def effective_push(preset: str, push: float) -> float:
    """image_pipeline.rs:369-375: the 1600 / caffenol stocks develop at least two stops."""
    p = preset.lower()
    return max(push, 2.0) if ("1600" in p or p == "caffenol") else max(push, 0.0)


def default_grain_px(preset: str, push: float = 0.0) -> float:
    """The CLI's grain size for a stock at 35 mm (main.rs:505-516)."""
    p = preset.lower()
    if p in ("t-max", "tmax"):
        return 1.1
    if p in ("hp5", "hp5-plus"):
        return 1.8
    if p in ("tri-x-1600", "trix-1600", "caffenol"):
        return 2.2
    return 2.2 if push >= 1.5 else 2.4


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _run(fn, *args):
    from .api import _check, _engine

    e = _engine(None)
    _check(e, getattr(e._lib, fn)(e._h, *args))


def blend_tiles(out_w: int, out_h: int, grid: list[Tile], step: int, pad: int, densities) -> np.ndarray:
    """Hann overlap blend of tile densities (grid order) into the image's d_norm."""
    desc = np.array([[t.tx, t.ty, t.x_start, t.y_start, t.tw, t.th] for t in grid], np.uint32).ravel()
    ds = [np.ascontiguousarray(d, np.float32) for d in densities]
    ptrs = (C.POINTER(C.c_float) * len(ds))(*[_fptr(d) for d in ds])
    out = np.zeros((out_h, out_w), np.float32)
    _run("fg_blend_tiles", out_w, out_h, step, pad, len(ds), desc.ctypes.data_as(C.POINTER(C.c_uint32)), ptrs,
         _fptr(out))
    return out


def scanner_otf(field, taps=None) -> np.ndarray:
    f = np.ascontiguousarray(field, np.float32)
    out = np.zeros_like(f)
    k = None if taps is None else np.ascontiguousarray(taps, np.float32)
    _run("fg_scanner_otf", _fptr(f), f.shape[1], f.shape[0], None if k is None else _fptr(k), _fptr(out))
    return out


def resize_triangle(field, ow: int, oh: int) -> np.ndarray:
    f = np.ascontiguousarray(field, np.float32)
    out = np.zeros((oh, ow), np.float32)
    _run("fg_resize_triangle", _fptr(f), f.shape[1], f.shape[0], ow, oh, _fptr(out))
    return out


# ---- whole images through the batched tile path ----

COLOR_SEED_OFFSETS = (0, 10007, 20011)  # R, G, B layer seeds (image_pipeline.rs:1048-1061, wrapping adds)


def image_tile_params(preset: str, grain_px: float, grid: list[Tile], exposure: float = 1.0, push: float = 0.0,
                      seed: int = 0) -> list:
    """Tile-worker parameters of every tile of one black-and-white image (pixel = 1 / grain_px um)."""
    from .api import tile_params

    return [tile_params(preset, 1.0 / grain_px, t.tw, t.th, exposure, push, tile_seed(seed, t)) for t in grid]


def render_tiles(params: list, tiles: list, engine=None, batch=None):
    """Renders exposure tiles (one batch, one graph launch) and returns their densities."""
    from .api import Batch

    b = batch or Batch(params, engine, use_graph=True, autotune=False)
    b.set_exposure(tiles)
    b.run()
    b.wait()
    out = b.density()
    if batch is None:
        b.close()
    return out


def render_bw_image(exposure, preset: str, grain_px: float, push: float = 0.0, seed: int = 0, engine=None):
    """render_film_black_and_white_tiled's tile path (image_pipeline.rs:377-649): tiles of the
    exposure image rendered in one batch and Hann-blended into the image's d_norm."""
    exposure = np.ascontiguousarray(exposure, np.float32)
    H, W = exposure.shape
    grid, step, pad = tile_grid(W, H, grain_px)
    params = image_tile_params(preset, grain_px, grid, 1.0, push, seed)
    tiles = [exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw] for t in grid]
    return blend_tiles(W, H, grid, step, pad, render_tiles(params, tiles, engine))


def render_color_image(rgb, preset: str, grain_px: float, push: float = 0.0, seed: int = 0, engine=None):
    """render_film_color_tiled (image_pipeline.rs:1017-1085): the R, G and B layers are independent
    black-and-white runs with seeds seed, seed + 10007 and seed + 20011; here all three channels'
    tiles share one batch.  Returns d_norm per channel, shape (3, H, W)."""
    rgb = np.ascontiguousarray(rgb, np.float32)
    H, W = rgb.shape[1:]
    grid, step, pad = tile_grid(W, H, grain_px)
    params, tiles = [], []
    for c, off in enumerate(COLOR_SEED_OFFSETS):
        params += image_tile_params(preset, grain_px, grid, 1.0, push, (seed + off) & M64)
        tiles += [np.ascontiguousarray(rgb[c, t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]) for t in grid]
    d = render_tiles(params, tiles, engine)
    n = len(grid)
    return np.stack([blend_tiles(W, H, grid, step, pad, d[c * n:(c + 1) * n]) for c in range(3)])
