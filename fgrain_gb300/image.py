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
