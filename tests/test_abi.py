"""The C ABI without a GPU: the library loads, exports every entry point include/fgrain_cuda.h
declares, its structs have the layouts ctypes assumes, and the preset table matches the
reference's presets (emulsion.rs:46-136)."""
import ctypes as C
import re
import subprocess
import textwrap
from pathlib import Path

import pytest

import fgrain_gb300 as fg
from fgrain_gb300 import _abi
from tests.helpers import REFERENCE_PRESETS

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fgrain_cuda.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(fg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported_and_bound():
    lib = _abi.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
        assert n in _abi.PROTOTYPES, f"{n} has no ctypes prototype"
    assert set(_abi.PROTOTYPES) == set(names)


STRUCTS = ["fg_optics", "fg_emulsion_cfg", "fg_exposure_cfg", "fg_dev_cfg", "fg_dev_report",
           "fg_scan_cfg", "fg_crystals_host", "fg_crystals_out", "fg_segment", "fg_timings",
           "fg_tile_params", "fg_batch_options", "fg_batch_stats", "fg_device_crystals", "fg_film_options",
           "fg_film_report", "fg_finish_cfg"]


def test_struct_layouts_match_ctypes(tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for s in STRUCTS:
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in getattr(_abi, s)._fields_:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for s in STRUCTS:
        ct = getattr(_abi, s)
        assert int(got[s]) == C.sizeof(ct), s
        for f, _ in ct._fields_:
            assert int(got[f"{s}.{f}"]) == getattr(ct, f).offset, f"{s}.{f}"


@pytest.mark.parametrize("name", list(REFERENCE_PRESETS))
def test_preset_table_matches_reference(name):
    cfg = fg.EmulsionConfig.preset(name, 33.0, 44.0)
    d, r, m, v, mo, ar, o, s = REFERENCE_PRESETS[name]
    assert cfg.dimensions == (33.0, 44.0, d)
    assert (cfg.r_min, cfg.mean_crystal_radius, cfg.size_variance, int(cfg.morphology), cfg.tabular_aspect_ratio,
            cfg.base_sensitivity) == (r, m, v, mo, ar, s)
    oo = cfg.optics
    assert (oo.refractive_index, oo.absorption_coeff, oo.scattering_coeff, oo.anisotropy_g,
            oo.antihalation_reflectance, oo.antihalation_density) == o


def test_unknown_preset_is_invalid_argument():
    with pytest.raises(fg.GpuError) as ei:
        fg.EmulsionConfig.preset("portra", 1.0, 1.0)
    assert ei.value.status == 16


def test_status_strings_mirror_gpu_error():
    lib = _abi.load()
    # error.rs:9-33 messages for the six GpuError variants.
    assert lib.fg_status_string(1).decode().startswith("Failed to find suitable GPU adapter")
    assert lib.fg_status_string(6).decode() == "GPU pipeline error"
    assert lib.fg_status_string(0).decode() == "ok"


def test_engine_creation_reports_status_without_crashing():
    lib = _abi.load()
    h = C.c_void_p()
    st = lib.fg_engine_create(0, C.byref(h))
    assert st in (0, 1)
    if st == 0:
        assert lib.fg_engine_destroy(h) == 0
    assert lib.fg_engine_create(-1, C.byref(h)) == 1
    assert lib.fg_engine_destroy(None) == 16


@pytest.mark.parametrize("preset,push", [("tri-x", 0.0), ("tri-x", 2.0), ("t-max", 1.0), ("hp5", 0.5),
                                         ("tri-x-1600", 0.0)])
def test_tile_params_follow_the_cpu_tile_worker(preset, push):
    """fg_tile_params_preset reproduces render_tile_cpu_full's configuration
    (image_pipeline.rs:925-1002) for every stock and push."""
    from tests.helpers import tile_worker_dev_cfg, REFERENCE_PRESETS
    px = 0.5
    p = fg.tile_params(preset, px, 100, 80, 0.7, push, 99)
    eff = max(push, 2.0) if "1600" in preset else max(push, 0.0)
    stock = preset if preset in ("t-max", "hp5", "tri-x-1600") else ("tri-x-1600" if eff >= 1.5 else "tri-x")
    d, r, m, v, mo, ar, o, sens = REFERENCE_PRESETS[stock]
    assert (p.film_w, p.film_h, p.film_d) == (50.0, 40.0, d)
    assert (p.r_min, p.mean_crystal_radius, p.size_variance, p.morphology, p.base_sensitivity) == (r, m, v, mo, sens)
    base = preset if preset in ("t-max", "hp5") else "tri-x"
    dc = tile_worker_dev_cfg(base, eff)
    assert p.threshold_photons == 4
    assert abs(p.filament_expansion - dc.filament_expansion) < 1e-15
    assert abs(p.clumping_proximity_factor - dc.clumping_proximity_factor) < 1e-15
    assert (p.samples_per_pixel, p.silver_opacity, p.seed) == (4, 0.25, 99)
    assert (p.photons_per_sq_um, p.illumination_angle_rad, p.crystal_absorption_coeff, p.max_bounces) == (6.0, 0.12, 1.3, 48)
    assert p.exposure == 0.7


def test_static_scan_rejects_misaligned_device_pointers_before_any_gpu_call():
    """fg_scan_crystals_static checks the alignment of every device array before it touches the
    GPU (so this runs without one): float4 arrays 16 bytes, FP64 arrays 8 bytes, out 4 bytes."""
    lib = _abi.load()
    cfg = fg.EmulsionConfig.preset("tri-x", 10.0, 10.0).to_c()
    scan = fg.ScanConfig(16, 16, 4, 0, 0.25).to_c()
    ok = 0x10000  # aligned stand-in addresses: never dereferenced, the checks fail first
    cases = [
        (dict(a=ok + 8), b"16-byte aligned"),
        (dict(pos64=ok + 4, dims64=ok, quat64=ok), b"8-byte aligned"),
        (dict(pos64=ok, dims64=ok, quat64=ok + 12), b"8-byte aligned"),
        (dict(expansion=ok + 2), b"8-byte aligned"),
        (dict(out=ok + 2), b"4-byte aligned"),
    ]
    for over, what in cases:
        f = dict(a=ok, q=ok, d=ok, pos64=None, dims64=None, quat64=None, developed=ok, expansion=ok, out=ok)
        f.update(over)
        dc = _abi.fg_device_crystals(f["a"], f["q"], f["d"], f["pos64"], f["dims64"], f["quat64"],
                                     f["developed"], f["expansion"], 1)
        msg = C.create_string_buffer(256)
        st = lib.fg_scan_crystals_static(C.byref(dc), C.byref(cfg), C.byref(scan), 1, f["out"], None, None,
                                         msg, len(msg))
        assert st == _abi.FG_ERR_INVALID_ARG and what in msg.value, (over, msg.value)
