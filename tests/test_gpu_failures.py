"""Failure detection without a GPU fault.  On a device error the reference falls back to its CPU
chain (image_pipeline.rs:535-558, gpu.rs:9-14); this library has no fallback: every entry point
returns a status (GpuError in Python) and the engine stays usable for the next call.  Each test
makes one failure on purpose, by host-side means only, and then renders normally on the same
engine:
  * a bounded device wait that runs out (a synthesis column also waits on a flag that nothing
    sets, with a short limit): FG_ERR_DEVICE_TIMEOUT;
  * a fixed device capacity exceeded (the scan's bin lists): FG_ERR_DEVICE_OVERFLOW;
  * an allocation refused (a process-wide device budget): FG_ERR_OOM;
  * truncated or missing tile lists: FG_ERR_INVALID_ARG before any device work.
"""
import ctypes as C

import numpy as np
import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import _abi

pytestmark = pytest.mark.gpu


def small_tile(seed=3):
    p = fg.tile_params("tri-x", 1 / 2.4, 64, 48, 1.0, 0.0, seed)
    return p, np.full((48, 64), 0.5, np.float32)


def renders_normally(engine):
    p, t = small_tile(9)
    d = fg.render_tile(t, p, engine)
    assert np.isfinite(d).all() and (d >= 0.05 - 1e-6).all()


def test_bounded_wait_runs_out_with_device_timeout(engine):
    p, t = small_tile()
    b = fg.Batch([p, p], engine, use_graph=False, synth_wait_limit=1000, wait_probe=True)
    b.set_exposure([t, t])
    with pytest.raises(fg.GpuError) as ei:
        b.run()
        b.wait()
    assert ei.value.status == _abi.FG_ERR_DEVICE_TIMEOUT and "bounded wait" in str(ei.value)
    b.close()
    renders_normally(engine)


def test_bin_list_overflow_is_reported(engine):
    """A filament expansion of 30 makes every developed crystal's leaf box span ~100 scan bins,
    past the batch's fixed list capacity (8 entries per crystal slot)."""
    p, t = small_tile(4)
    p.filament_expansion = 30.0
    b = fg.Batch([p], engine, use_graph=False)
    b.set_exposure([t])
    with pytest.raises(fg.GpuError) as ei:
        b.run()
        b.wait()
    assert ei.value.status == _abi.FG_ERR_DEVICE_OVERFLOW and "work list overflow" in str(ei.value)
    b.close()
    renders_normally(engine)


def test_device_budget_refuses_allocation(engine):
    lib = _abi.load()
    p, t = small_tile(5)
    try:
        assert lib.fg_set_device_budget(1 << 16) == _abi.FG_OK
        with pytest.raises(fg.GpuError) as ei:
            fg.render_tile(t, p, engine)
        assert ei.value.status == _abi.FG_ERR_OOM and "budget" in str(ei.value)
    finally:
        lib.fg_set_device_budget(0)
    renders_normally(engine)


def test_truncated_tile_lists_are_rejected(engine):
    lib = _abi.load()
    p, t = small_tile(6)
    b = fg.Batch([p, p], engine, use_graph=False)
    fp = t.ctypes.data_as(C.POINTER(C.c_float))
    half = (C.POINTER(C.c_float) * 2)(fp, None)  # the second tile is missing
    assert lib.fg_batch_set_exposure(b._h, half) == _abi.FG_ERR_INVALID_ARG
    assert lib.fg_batch_set_exposure(b._h, None) == _abi.FG_ERR_INVALID_ARG
    assert lib.fg_batch_get_density(b._h, None) == _abi.FG_ERR_INVALID_ARG
    ptr = C.POINTER(C.c_float)()
    assert lib.fg_batch_exposure_device(b._h, 2, C.byref(ptr)) == _abi.FG_ERR_INVALID_ARG
    h = C.c_void_p()
    assert lib.fg_batch_create(engine._h, None, 0, None, C.byref(h)) == _abi.FG_ERR_INVALID_ARG
    arr = (_abi.fg_tile_params * 1)(p)
    assert lib.fg_render_batch(engine._h, arr, 0, None, None) == _abi.FG_ERR_INVALID_ARG
    # the batch is intact: the full list renders, and equals the plain path
    b.set_exposure([t, t])
    b.run()
    b.wait()
    out = b.density()
    np.testing.assert_array_equal(out[0], fg.render_tile(t, p, engine))
    b.close()
