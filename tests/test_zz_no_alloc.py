"""GPU test of fg_scan_crystals_static, the scan entry point that allocates no device memory.

Some callers cannot let a library allocate device memory: a host that owns a fixed device-memory
budget or its own pool allocator, or a plugin inside one.  They hand over the crystals and the
output image in device memory they already hold (here torch tensors stand in for such a pool).
Two calls in a row, with different crystal sets, image sizes, strata and modes, must each give
exactly the image of fg_scan_emulsion on the same crystals (same kernels, same staging, fixed-point
chord sums): the second call starts from the scratch contents the first one left behind.  The
file name makes pytest collect it last; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import _abi
from oracle import oracle as orc
from tests.helpers import reference_cfg

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5  # the scan parity tolerance (relative transmittance)


def developed_crystals(preset, w, h, seed, float_exact):
    """Oracle-synthesized crystals with oracle development of random latent counts."""
    cfg = reference_cfg(preset, w, h)
    cr = orc.synthesize(cfg, seed)
    if float_exact:  # values the float arrays hold exactly, so no FP64 copies are needed
        for k in ("pos", "dims", "quat", "sens"):
            setattr(cr, k, getattr(cr, k).astype(np.float32).astype(np.float64))
    rng = np.random.default_rng(seed)
    cr.latent[:] = rng.integers(0, 12, len(cr)).astype(np.uint32)
    orc.develop(cr, fg.DevelopmentConfig(4, 1.2, 1.5, 0.85))
    assert 0 < cr.developed.sum() < len(cr)
    return cfg, cr


def reference_scan(engine, cfg, cr, scan, seed):
    em = fg.VirtualEmulsionLayer.from_crystals(cfg, cr.pos, cr.dims, cr.quat, cr.sens, cr.morph, engine)
    em.set_development(cr.developed, cr.expansion)
    out, img = fg.scan_emulsion(em, scan, seed)
    em.close()
    return out, img


def static_scan(torch, cfg, cr, scan, seed, with64):
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to("cuda")  # noqa: E731
    a = dev(np.concatenate([cr.pos, cr.sens[:, None]], axis=1).astype(np.float32))
    q = dev(cr.quat.astype(np.float32))
    d = dev(np.concatenate([cr.dims.astype(np.float32), cr.morph.view(np.float32)[:, None]], axis=1))
    keep = [a, q, d, dev(cr.developed), dev(cr.expansion)]
    p64 = [None, None, None]
    if with64:
        keep += [dev(cr.pos), dev(cr.dims), dev(cr.quat)]
        p64 = [t.data_ptr() for t in keep[5:]]
    dc = _abi.fg_device_crystals(a.data_ptr(), q.data_ptr(), d.data_ptr(), p64[0], p64[1], p64[2],
                                 keep[3].data_ptr(), keep[4].data_ptr(), len(cr))
    out = torch.full((scan.height_px, scan.width_px), -1.0, dtype=torch.float32, device="cuda")
    img = torch.zeros((scan.height_px, scan.width_px), dtype=torch.uint8, device="cuda")
    msg = C.create_string_buffer(512)
    torch.cuda.synchronize()
    st = _abi.load().fg_scan_crystals_static(C.byref(dc), C.byref(cfg.to_c()), C.byref(scan.to_c()),
                                             seed, out.data_ptr(), img.data_ptr(), None, msg, len(msg))
    assert st == _abi.FG_OK, (_abi.STATUS_NAMES.get(st), msg.value.decode())
    return out.cpu().numpy(), img.cpu().numpy()


def test_static_scan_matches_scan_emulsion_twice(engine):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    calls = [
        # (preset, film um, scan config, seed, FP64 copies)
        ("tri-x", (40.0, 32.0), fg.ScanConfig(96, 80, 4, 0, 0.25), 5, True),
        ("hp5", (24.0, 30.0), fg.ScanConfig(40, 50, 9, 2, 0.4), 6, False),
    ]
    for preset, (w, h), scan, seed, with64 in calls:
        cfg, cr = developed_crystals(preset, w, h, seed, float_exact=not with64)
        ref_out, ref_img = reference_scan(engine, cfg, cr, scan, seed)
        out, img = static_scan(torch, cfg, cr, scan, seed, with64)
        assert (out >= 0).all()
        # The same image bit for bit (the scan tolerance would allow T_RTOL).
        np.testing.assert_array_equal(out, ref_out)
        np.testing.assert_array_equal(img, ref_img)
        assert (ref_out < 0.999).mean() > 0.05  # the developed crystals do shade the image


def test_static_scan_rejects_requests_beyond_its_scratch(engine):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    dc = _abi.fg_device_crystals(None, None, None, None, None, None, None, None, 0)
    scan = fg.ScanConfig(2048, 2048, 4, 0, 0.25)  # 256 x 256 bins of 8 px
    out = torch.full((8,), -1.0, dtype=torch.float32, device="cuda")
    msg = C.create_string_buffer(512)
    st = _abi.load().fg_scan_crystals_static(C.byref(dc), C.byref(cfg.to_c()), C.byref(scan.to_c()), 1,
                                             out.data_ptr(), None, None, msg, len(msg))
    assert st == _abi.FG_ERR_INVALID_ARG and b"at most 16384" in msg.value, msg.value
    assert (out.cpu().numpy() == -1.0).all()


def test_static_scan_rejects_more_bin_entries_than_its_scratch(engine):
    """100 developed cubes that each cover the whole film make 100 x 16384 (crystal, bin) entries,
    more than the scratch's 1,048,576: the call fails after counting and leaves out untouched."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    cfg = reference_cfg("tri-x", 20.0, 20.0)
    n = 100
    rng = np.random.default_rng(3)
    pos = np.column_stack([10.0 + rng.random(n), 10.0 + rng.random(n), np.full(n, 7.0)])
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to("cuda")  # noqa: E731
    a = dev(np.column_stack([pos, np.ones(n)]).astype(np.float32))
    q = dev(np.tile(np.array([0.0, 0.0, 0.0, 1.0], np.float32), (n, 1)))
    d = dev(np.column_stack([np.full((n, 3), 11.0, np.float32), np.zeros(n, np.int32).view(np.float32)]))
    developed = dev(np.ones(n, np.uint8))
    expansion = dev(np.ones(n))
    dc = _abi.fg_device_crystals(a.data_ptr(), q.data_ptr(), d.data_ptr(), None, None, None,
                                 developed.data_ptr(), expansion.data_ptr(), n)
    scan = fg.ScanConfig(1024, 1024, 4, 0, 0.25)  # 128 x 128 bins of 8 px: exactly the bin limit
    out = torch.full((1024, 1024), -1.0, dtype=torch.float32, device="cuda")
    msg = C.create_string_buffer(512)
    st = _abi.load().fg_scan_crystals_static(C.byref(dc), C.byref(cfg.to_c()), C.byref(scan.to_c()), 1,
                                             out.data_ptr(), None, None, msg, len(msg))
    assert st == _abi.FG_ERR_INVALID_ARG and b"at most 1048576" in msg.value, msg.value
    assert (out.cpu().numpy() == -1.0).all()
