"""Fast-approximation mode: the reference's wgpu tile model (GpuEngine::render_tile_all_gpu,
gpu.rs:491-938, and its poisson / develop / scan shaders) on the device, over the C ABI's
fg_render_tiles_fast.  A different, cheaper model than the CPU-path physics of render_tile."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi

CELL_DTYPE = np.dtype([("pos", "<f4", 4), ("dims_exp", "<f4", 4), ("rot", "<f4", 4), ("flags", "<u4", 4)])


def tile_params_fast(preset: str, pixel_size_um: float, tw: int, th: int, exposure: float = 1.0,
                     push: float = 0.0, tile_seed: int = 0) -> _abi.fg_tile_params:
    """GpuTileParams of the reference's GPU branch (image_pipeline.rs:455-518)."""
    from .api import _check

    p = _abi.fg_tile_params()
    _check(None, _abi.load().fg_tile_params_fast_preset(preset.encode(), pixel_size_um, tw, th, exposure, push,
                                                        tile_seed & 0xFFFFFFFFFFFFFFFF, C.byref(p)))
    return p


def fast_grid(params: _abi.fg_tile_params):
    """((w, h, d), cell_size) of the tile's cell grid (gpu.rs:505-525)."""
    dims = (C.c_uint32 * 3)()
    cs = C.c_float()
    _abi.load().fg_fast_grid(C.byref(params), dims, C.byref(cs))
    return tuple(dims), cs.value


def render_tiles_fast(params: list, tiles: list, engine=None, cells: bool = False):
    """d_neg of every tile (one set of launches); with cells=True also each tile's final grid as a
    (d, h, w) array of CELL_DTYPE records."""
    from .api import _check, _engine

    e = _engine(engine)
    n = len(params)
    ts = [np.ascontiguousarray(t, np.float32) for t in tiles]
    outs = [np.zeros((p.height_px, p.width_px), np.float32) for p in params]
    grids = []
    if cells:
        for p in params:
            (w, h, d), _ = fast_grid(p)
            grids.append(np.zeros((d, h, w), CELL_DTYPE))
    P = (_abi.fg_tile_params * n)(*params)
    fp = C.POINTER(C.c_float)
    tp = (fp * n)(*[t.ctypes.data_as(fp) for t in ts])
    op = (fp * n)(*[o.ctypes.data_as(fp) for o in outs])
    cp = (C.c_void_p * n)(*[g.ctypes.data for g in grids]) if cells else None
    _check(e, e._lib.fg_render_tiles_fast(e._h, P, n, tp, op, cp))
    return (outs, grids) if cells else outs


def render_tile_fast(tile, params: _abi.fg_tile_params, engine=None, cells: bool = False):
    r = render_tiles_fast([params], [tile], engine, cells)
    return (r[0][0], r[1][0]) if cells else r[0]
