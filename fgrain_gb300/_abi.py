"""ctypes view of include/fgrain_cuda.h.

The structures below mirror the C declarations field for field; every function prototype is
declared so that ctypes checks argument types.  Loading fails loudly when the shared library has
not been built: there is no Python or CPU fallback for the path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfgrain_cuda.so"

FG_OK = 0
STATUS_NAMES = {
    0: "FG_OK",
    1: "FG_ERR_ADAPTER_NOT_FOUND",
    2: "FG_ERR_DEVICE_REQUEST_FAILED",
    3: "FG_ERR_CHANNEL",
    4: "FG_ERR_BUFFER_MAP",
    5: "FG_ERR_BUFFER_RANGE",
    6: "FG_ERR_PIPELINE",
    16: "FG_ERR_INVALID_ARG",
    17: "FG_ERR_OOM",
    18: "FG_ERR_DEVICE_TIMEOUT",
    19: "FG_ERR_DEVICE_OVERFLOW",
}
globals().update({name: code for code, name in STATUS_NAMES.items()})  # FG_ERR_INVALID_ARG = 16, ...


class fg_optics(C.Structure):
    _fields_ = [("refractive_index", C.c_double), ("absorption_coeff", C.c_double),
                ("scattering_coeff", C.c_double), ("anisotropy_g", C.c_double),
                ("antihalation_reflectance", C.c_double), ("antihalation_density", C.c_double)]


class fg_emulsion_cfg(C.Structure):
    _fields_ = [("width", C.c_double), ("height", C.c_double), ("depth", C.c_double),
                ("r_min", C.c_double), ("mean_crystal_radius", C.c_double),
                ("size_variance", C.c_double), ("morphology", C.c_int32), ("_pad", C.c_int32),
                ("tabular_aspect_ratio", C.c_double), ("optics", fg_optics),
                ("base_sensitivity", C.c_double)]


class fg_exposure_cfg(C.Structure):
    _fields_ = [("photons_per_sq_um", C.c_double), ("illumination_angle_rad", C.c_double),
                ("crystal_absorption_coeff", C.c_double), ("max_bounces", C.c_uint32),
                ("_pad", C.c_uint32)]


class fg_dev_cfg(C.Structure):
    _fields_ = [("threshold_photons", C.c_uint32), ("_pad", C.c_uint32),
                ("filament_expansion", C.c_double), ("clumping_proximity_factor", C.c_double),
                ("developer_contrast", C.c_double)]


class fg_dev_report(C.Structure):
    _fields_ = [("total_crystals", C.c_uint64), ("developed_crystals", C.c_uint64),
                ("fixed_crystals", C.c_uint64), ("total_clumps", C.c_uint64),
                ("max_clump_size", C.c_uint64), ("avg_clump_size", C.c_double)]


class fg_scan_cfg(C.Structure):
    _fields_ = [("width_px", C.c_uint32), ("height_px", C.c_uint32),
                ("samples_per_pixel", C.c_uint32), ("mode", C.c_int32),
                ("silver_opacity", C.c_double)]


_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class fg_crystals_host(C.Structure):
    _fields_ = [("pos", _dp), ("dims", _dp), ("quat", _dp), ("sensitivity", _dp),
                ("morphology", _ip)]


class fg_crystals_out(C.Structure):
    _fields_ = [("pos", _dp), ("dims", _dp), ("quat", _dp), ("sensitivity", _dp),
                ("morphology", _ip)]


class fg_segment(C.Structure):
    _fields_ = [("origin", C.c_double * 3), ("dir", C.c_double * 3), ("step", C.c_double),
                ("energy", C.c_double), ("photon", C.c_uint32), ("bounce", C.c_uint32)]


class fg_timings(C.Structure):
    _fields_ = [("synth_ms", C.c_double), ("bvh_ms", C.c_double), ("transport_ms", C.c_double),
                ("develop_ms", C.c_double), ("scan_ms", C.c_double), ("post_ms", C.c_double),
                ("total_ms", C.c_double), ("crystals", C.c_uint64), ("photons", C.c_uint64),
                ("hits", C.c_uint64), ("rays", C.c_uint64), ("developed", C.c_uint64),
                ("fallbacks", C.c_uint64), ("kernel_launches", C.c_uint32),
                ("error_word", C.c_uint32)]


class fg_tile_params(C.Structure):
    _fields_ = [("film_w", C.c_double), ("film_h", C.c_double), ("film_d", C.c_double),
                ("width_px", C.c_uint32), ("height_px", C.c_uint32),
                ("samples_per_pixel", C.c_uint32), ("threshold_photons", C.c_uint32),
                ("silver_opacity", C.c_double), ("seed", C.c_uint64),
                ("r_min", C.c_double), ("mean_crystal_radius", C.c_double), ("size_variance", C.c_double),
                ("morphology", C.c_int32), ("_pad0", C.c_int32),
                ("tabular_aspect_ratio", C.c_double), ("base_sensitivity", C.c_double),
                ("exposure", C.c_double), ("filament_expansion", C.c_double),
                ("clumping_proximity_factor", C.c_double), ("optics", fg_optics),
                ("photons_per_sq_um", C.c_double), ("illumination_angle_rad", C.c_double),
                ("crystal_absorption_coeff", C.c_double), ("max_bounces", C.c_uint32),
                ("_pad1", C.c_uint32)]


class fg_batch_options(C.Structure):
    _fields_ = [("use_graph", C.c_int32), ("autotune", C.c_int32), ("transport_threads", C.c_uint32),
                ("transport_blocks", C.c_uint32), ("scan_bin_px", C.c_uint32), ("synth_wait_limit", C.c_uint32),
                ("wait_probe", C.c_int32), ("_pad", C.c_uint32)]


class fg_batch_stats(C.Structure):
    _fields_ = [("synth_ms", C.c_double), ("bvh_ms", C.c_double), ("transport_ms", C.c_double),
                ("develop_ms", C.c_double), ("scan_ms", C.c_double), ("total_ms", C.c_double),
                ("crystals", C.c_uint64), ("photons", C.c_uint64), ("rays", C.c_uint64),
                ("pixels", C.c_uint64), ("hits", C.c_uint64), ("scan_hits", C.c_uint64),
                ("scan_fallbacks", C.c_uint64), ("transport_threads", C.c_uint32),
                ("transport_blocks", C.c_uint32), ("scan_bin_px", C.c_uint32), ("graph", C.c_uint32),
                ("kernel_launches", C.c_uint32), ("_pad", C.c_uint32), ("developed", C.c_uint64),
                ("clumps", C.c_uint64), ("cells", C.c_uint64), ("bridson_ms", C.c_double)]


class fg_device_crystals(C.Structure):
    _fields_ = [("a", C.c_void_p), ("q", C.c_void_p), ("d", C.c_void_p), ("pos64", C.c_void_p),
                ("dims64", C.c_void_p), ("quat64", C.c_void_p), ("developed", C.c_void_p),
                ("expansion", C.c_void_p), ("n", C.c_uint64)]


class fg_film_options(C.Structure):
    _fields_ = [("preset", C.c_char_p), ("grain_size_px", C.c_double), ("grain_strength", C.c_double),
                ("exposure", C.c_double), ("color", C.c_int32), ("out_w", C.c_uint32), ("out_h", C.c_uint32),
                ("tile_size", C.c_uint32), ("seed", C.c_uint64), ("auto_scale", C.c_int32),
                ("reference_res", C.c_uint32), ("scale", C.c_double), ("supersample", C.c_uint32),
                ("scanner_otf", C.c_int32), ("push", C.c_double), ("eberhard", C.c_double),
                ("batch_bytes", C.c_uint64)]


class fg_film_report(C.Structure):
    _fields_ = [("in_w", C.c_uint32), ("in_h", C.c_uint32), ("out_w", C.c_uint32), ("out_h", C.c_uint32),
                ("total_tiles", C.c_uint64), ("total_crystals", C.c_uint64), ("photons", C.c_uint64),
                ("elapsed_seconds", C.c_double), ("developed_crystals", C.c_uint64),
                ("total_clumps", C.c_uint64), ("prep_ms", C.c_double), ("tiles_ms", C.c_double),
                ("finish_ms", C.c_double)]


class fg_finish_cfg(C.Structure):
    _fields_ = [("preset", C.c_char_p), ("grain_size_px", C.c_double), ("grain_strength", C.c_double),
                ("push", C.c_double), ("scanner_otf", C.c_int32), ("_pad", C.c_int32)]


_vp = C.c_void_p
_st = C.c_int
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_u16p = C.POINTER(C.c_uint16)
_i64p = C.POINTER(C.c_int64)
_fp = C.POINTER(C.c_float)
_szp = C.POINTER(C.c_size_t)

# name -> (restype, argtypes); the complete list of entry points in include/fgrain_cuda.h.
PROTOTYPES = {
    "fg_engine_create": (_st, [C.c_int, C.POINTER(_vp)]),
    "fg_engine_destroy": (_st, [_vp]),
    "fg_last_error": (C.c_char_p, [_vp]),
    "fg_engine_device_name": (C.c_char_p, [_vp]),
    "fg_engine_timings": (_st, [_vp, C.POINTER(fg_timings)]),
    "fg_status_string": (C.c_char_p, [_st]),
    "fg_emulsion_preset": (_st, [C.c_char_p, C.c_double, C.c_double, C.POINTER(fg_emulsion_cfg)]),
    "fg_emulsion_upload": (_st, [_vp, C.POINTER(fg_emulsion_cfg), C.POINTER(fg_crystals_host),
                                 C.c_size_t, C.POINTER(_vp)]),
    "fg_emulsion_synthesize": (_st, [_vp, C.POINTER(fg_emulsion_cfg), C.c_uint64, C.POINTER(_vp)]),
    "fg_emulsion_destroy": (_st, [_vp, _vp]),
    "fg_emulsion_count": (_st, [_vp, _szp]),
    "fg_emulsion_download": (_st, [_vp, _vp, C.POINTER(fg_crystals_out)]),
    "fg_emulsion_get_counts": (_st, [_vp, _vp, _u32p]),
    "fg_emulsion_set_counts": (_st, [_vp, _vp, _u32p]),
    "fg_emulsion_get_development": (_st, [_vp, _vp, _u8p, _i64p, _dp]),
    "fg_emulsion_set_development": (_st, [_vp, _vp, _u8p, _dp]),
    "fg_expose_emulsion": (_st, [_vp, _vp, _fp, C.c_uint32, C.c_uint32,
                                 C.POINTER(fg_exposure_cfg), C.c_uint64]),
    "fg_develop_emulsion": (_st, [_vp, _vp, C.POINTER(fg_dev_cfg), C.POINTER(fg_dev_report)]),
    "fg_scan_emulsion": (_st, [_vp, _vp, C.POINTER(fg_scan_cfg), C.c_uint64, _fp, _fp, _u8p]),
    "fg_replay_segments": (_st, [_vp, _vp, C.POINTER(fg_exposure_cfg), C.c_uint64,
                                 C.POINTER(fg_segment), C.c_size_t, _u32p, _u32p, C.c_size_t,
                                 _szp]),
    "fg_replay_rays": (_st, [_vp, _vp, _dp, _dp, C.c_size_t, C.c_int, _u32p, _u32p,
                             C.c_size_t, _szp, _dp]),
    "fg_scan_ray_hits": (_st, [_vp, _vp, C.POINTER(fg_scan_cfg), C.c_uint64, _u16p]),
    "fg_set_device_budget": (_st, [C.c_uint64]),
    "fg_emulsion_reference_tree": (_st, [_vp, _vp, C.c_int, _u32p, _u32p, _dp, C.c_size_t, _szp, _szp]),
    "fg_blend_tiles": (_st, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _u32p,
                             C.POINTER(_fp), _fp]),
    "fg_scanner_otf": (_st, [_vp, _fp, C.c_uint32, C.c_uint32, _fp, _fp]),
    "fg_resize_triangle": (_st, [_vp, _fp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _fp]),
    "fg_tile_params_fast_preset": (_st, [C.c_char_p, C.c_double, C.c_uint32, C.c_uint32, C.c_double,
                                         C.c_double, C.c_uint64, C.POINTER(fg_tile_params)]),
    "fg_fast_grid": (_st, [C.POINTER(fg_tile_params), _u32p, _fp]),
    "fg_render_tiles_fast": (_st, [_vp, C.POINTER(fg_tile_params), C.c_uint32, C.POINTER(_fp), C.POINTER(_fp),
                                   C.POINTER(_vp)]),
    "fg_render_tile_fast": (_st, [_vp, _fp, C.POINTER(fg_tile_params), _fp, _vp]),
    "fg_film_options_default": (None, [C.POINTER(fg_film_options)]),
    "fg_film_output_size": (_st, [C.POINTER(fg_film_options), C.c_uint32, C.c_uint32, _u32p, _u32p]),
    "fg_render_film": (_st, [_vp, _u8p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(fg_film_options), _u8p,
                             C.POINTER(fg_film_report)]),
    "fg_panchromatic_luma": (_st, [_vp, _u8p, C.c_uint32, C.c_uint32, C.c_char_p, _u8p]),
    "fg_resize_u8": (_st, [_vp, _u8p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32, _u8p]),
    "fg_gelatin_psf": (_st, [_vp, _u8p, C.c_uint32, C.c_uint32, _fp, _u32p]),
    "fg_film_finish": (_st, [_vp, C.POINTER(fg_finish_cfg), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                             C.c_uint32, _u32p, C.POINTER(_fp), _u8p, _fp, _u8p, _fp, _fp]),
    "fg_scan_signal": (_st, [_vp, _vp, C.POINTER(fg_scan_cfg), C.c_uint64, _fp, C.c_double, C.c_double, _fp, _fp]),
    "fg_scan_backward": (_st, [_vp, _vp, C.POINTER(fg_scan_cfg), C.c_uint64, _fp, C.c_double, C.c_double, _fp, _fp,
                               _dp, _dp]),
    "fg_tile_params_preset": (_st, [C.c_char_p, C.c_double, C.c_uint32, C.c_uint32, C.c_double,
                                    C.c_double, C.c_uint64, C.POINTER(fg_tile_params)]),
    "fg_render_tile": (_st, [_vp, _fp, C.POINTER(fg_tile_params), _fp]),
    "fg_batch_create": (_st, [_vp, C.POINTER(fg_tile_params), C.c_uint32, C.POINTER(fg_batch_options),
                              C.POINTER(_vp)]),
    "fg_batch_destroy": (_st, [_vp]),
    "fg_batch_set_exposure": (_st, [_vp, C.POINTER(_fp)]),
    "fg_batch_exposure_device": (_st, [_vp, C.c_uint32, C.POINTER(_fp)]),
    "fg_batch_density_device": (_st, [_vp, C.c_uint32, C.POINTER(_fp)]),
    "fg_batch_run": (_st, [_vp]),
    "fg_batch_wait": (_st, [_vp, C.POINTER(fg_batch_stats)]),
    "fg_batch_get_density": (_st, [_vp, C.POINTER(_fp)]),
    "fg_batch_tile_crystals": (_st, [_vp, C.c_uint32, C.POINTER(fg_crystals_out), _u32p, _u8p, _dp,
                                     C.c_size_t, _szp]),
    "fg_batch_time": (_st, [_vp, C.c_uint32, _dp]),
    "fg_host_alloc": (_st, [C.c_size_t, C.POINTER(_vp)]),
    "fg_host_free": (_st, [_vp]),
    "fg_render_batch": (_st, [_vp, C.POINTER(fg_tile_params), C.c_uint32, C.POINTER(_fp), C.POINTER(_fp)]),
    "fg_scan_crystals_static": (_st, [C.POINTER(fg_device_crystals), C.POINTER(fg_emulsion_cfg),
                                      C.POINTER(fg_scan_cfg), C.c_uint64, _vp, _vp, _vp, C.c_char_p,
                                      C.c_size_t]),
    "fg_png_unfilter": (_st, [_vp, C.c_uint32, C.c_uint32, C.c_uint32]),
    "fg_jpeg_info": (_st, [_vp, C.c_size_t, _u32p, _u32p, _u32p, C.c_char_p, C.c_size_t]),
    "fg_jpeg_decode": (_st, [_vp, C.c_size_t, _vp, C.c_size_t, C.c_char_p, C.c_size_t]),
    "fg_jpeg_encode": (_st, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_size_t,
                             C.POINTER(C.c_size_t)]),
    "fg_webp_info": (_st, [_vp, C.c_size_t, _u32p, _u32p, _u32p, C.c_char_p, C.c_size_t]),
    "fg_webp_decode": (_st, [_vp, C.c_size_t, _vp, C.c_size_t, C.c_char_p, C.c_size_t]),
    "fg_webp_encode": (_st, [_vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _vp, C.c_size_t,
                             C.POINTER(C.c_size_t)]),
}

# Options of the JPEG encoder (the FG_JPEG_* bits; a restart interval of n MCUs is n << 16).
FG_JPEG_SUBSAMPLE_420 = 0x0
FG_JPEG_SUBSAMPLE_422 = 0x1
FG_JPEG_SUBSAMPLE_444 = 0x2
FG_JPEG_SEPARATE_SCANS = 0x4


def FG_JPEG_RESTART(n: int) -> int:
    return n << 16


# Tools of the lossless WebP encoder (the FG_WEBP_* bits).
FG_WEBP_SUBTRACT_GREEN = 0x01
FG_WEBP_PREDICTOR = 0x02
FG_WEBP_COLOR_TRANSFORM = 0x04
FG_WEBP_PALETTE = 0x08
FG_WEBP_COLOR_CACHE = 0x10
FG_WEBP_BACKREFS = 0x20
FG_WEBP_META_CODES = 0x40
FG_WEBP_ALL_MODES = 0x80
FG_WEBP_DEFAULT = FG_WEBP_SUBTRACT_GREEN | FG_WEBP_PREDICTOR | FG_WEBP_COLOR_CACHE | FG_WEBP_BACKREFS

_lib = None


def load() -> C.CDLL:
    """Loads libfgrain_cuda.so (built by fgrain_gb300.build) and declares every prototype."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the fgrain GB300 path has no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
