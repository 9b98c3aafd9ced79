"""The ``fgrain`` command line (src/main.rs:12-1090) over the device renderer.

``python -m fgrain_gb300 <command> ...`` takes the reference binary's commands, options, defaults
and error messages: ``apply`` (also reached by giving an image path first) renders a photograph
through ``render_film``; ``gradient``, ``tri-x``, ``t-max``, ``halation`` and ``demo <name>``
run the demonstrations on one emulsion patch through the engine entry points (synthesize, expose,
develop, scan).  Everything runs on the GPU: ``--gpu`` is accepted and changes nothing.

``run_cli(argv)`` returns normally on success and raises ``CliError`` with the reference's
message otherwise; ``main`` prints ``error: <message>`` and exits 1, as ``main.rs:12-19`` does.
Image files are read and written by ``fgrain_gb300.imageio`` (PNG, PGM, PPM).
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

from . import imageio


class CliError(Exception):
    pass


def is_image_file(path: str) -> bool:
    """main.rs:88-94: the extensions that make a first argument an input image."""
    return path.lower().endswith((".png", ".jpg", ".jpeg", ".webp"))


# ---- help (main.rs:97-254) ----

_MAIN_HELP = """fgrain: physically based film grain simulation (GB300 device renderer)

Usage:
  fgrain <command> [arguments] [options]
  fgrain <input_image> [output_image] [options]

Commands:
  apply <input> [output]    Apply physically based film grain to an image
  gradient [output]         Render the continuous exposure ramp demonstration
  tri-x [output]            Render the Kodak Tri-X 400 preset demonstration
  t-max [output]            Render the Kodak T-Max 100 tabular grain demonstration
  halation [output]         Render the point-source halation demonstration
  demo <name> [output]      Run a demonstration (gradient, tri-x, t-max, halation)
  help [command]            Print this message or help for a given command

Options:
  -h, --help                Print help information

Run 'fgrain apply --help' for image processing options."""

_APPLY_HELP = """fgrain apply: apply physically based film grain to an input image

Usage:
  fgrain apply <input_image> [output_image] [options]
  fgrain <input_image> [output_image] [options]

Supported formats:
  PNG (.png); binary PGM and PPM (.pgm, .ppm). JPEG and WebP have no codec in this build.

Arguments:
  <input_image>                 Path to the input image file
  [output_image]                Path to the output image file (default: film_grained_output.png)

Options:
  -o, --output <path>           Output image path
  -p, --preset <stock>          Emulsion stock: tri-x, tri-x-1600, caffenol, t-max, hp5 (default: tri-x)
  -f, --format <format>         Negative format: 35mm, 120, 4x5 (default: 35mm)
      --push <stops>            Push processing stops, 0.0 to 3.0 (default: 0.0; 2.0 for tri-x-1600/caffenol)
      --eberhard <float>        Eberhard / Mackie adjacency strength (default: 0.0)
      --no-scanner-otf          Disable the scanner lens MTF
  -c, --color                   Simulate colour film dye clouds (RGB)
  -e, --exposure <float>        Exposure multiplier (default: 1.0)
  -s, --grain-size <pixels>     Crystal grain diameter in pixels (default: 2.4 for 35mm Tri-X)
      --grain-strength <float>  Grain contrast multiplier (default: 1.0)
      --scale <float>           Global grain scale multiplier (default: 1.0)
      --auto-scale              Scale grain size and strength relative to a 24 MP 35mm scan
      --reference-res <pixels>  Long edge of the reference scan for --auto-scale (default: 6000)
      --supersample <1-4>       Optical aperture supersampling factor (default: 1)
      --tile-size <pixels>      Processing tile edge (default: 320)
  -w, --width <pixels>          Output width (default: the input's)
      --height <pixels>         Output height (default: the input's)
      --gpu                     Accepted for compatibility: every stage already runs on the GPU
  -h, --help                    Print help information"""

_DEMO_HELP = """fgrain demo: run the film grain demonstrations

Usage:
  fgrain demo <gradient|tri-x|t-max|halation> [output_image] [options]
  fgrain <gradient|tri-x|t-max|halation> [output_image] [options]

Demonstrations:
  gradient    Continuous exposure ramp from shadow to highlight
  tri-x       Kodak Tri-X 400 cubic grain emulsion
  t-max       Kodak T-Max 100 tabular grain emulsion
  halation    Sub-surface scattering and anti-halation reflection

Options:
  -o, --output <path>  Output image path
  -h, --help           Print help information"""

_DEMO_TITLES = {"gradient": "Render the continuous exposure ramp demonstration",
                "tri-x": "Render the Kodak Tri-X 400 preset demonstration",
                "t-max": "Render the Kodak T-Max 100 tabular grain demonstration",
                "halation": "Render the point-source halation demonstration"}


def _demo_help(name: str) -> str:
    return (f"fgrain {name}: {_DEMO_TITLES[name]}\n\nUsage:\n  fgrain {name} [output_image] [options]\n\n"
            f"Arguments:\n  [output_image]       Output filename (default: film_grain_{name}.png)\n\n"
            "Options:\n  -o, --output <path>  Output image path\n  -h, --help           Print help information")


_HELP = {"apply": _APPLY_HELP, "image": _APPLY_HELP, "demo": _DEMO_HELP,
         **{k: _demo_help(k) for k in _DEMO_TITLES}}


# ---- dispatch (main.rs:21-86) ----

def run_cli(argv: list[str], out=None) -> None:
    """argv[0] is the program name, as in the reference's ``run_cli``."""
    say = (lambda s="": print(s, file=out)) if out else print
    if len(argv) <= 1:
        say(_MAIN_HELP)
        return
    first, rest = argv[1], argv[2:]
    if first in ("-h", "--help", "help"):
        if rest:
            topic = rest[0]
            if topic in _HELP:
                say(_HELP[topic])
            elif first == "help":
                raise CliError(f"unknown help topic '{topic}'. For a list of commands, try 'fgrain --help'.")
            else:
                say(_MAIN_HELP)
        else:
            say(_MAIN_HELP)
        return
    if first in ("apply", "image"):
        return run_image_apply(rest, say)
    if first in _DEMO_TITLES:
        return _run_demo_cli(first, rest, say)
    if first == "demo":
        if not rest or any(a in ("-h", "--help") for a in rest):
            say(_DEMO_HELP)
            return
        if rest[0] not in _DEMO_TITLES:
            raise CliError(f"unknown demo '{rest[0]}'. Available demos: gradient, tri-x, t-max, halation.\n"
                           "For more information, try 'fgrain demo --help'.")
        return _run_demo_cli(rest[0], rest[1:], say)
    if is_image_file(first):
        return run_image_apply(argv[1:], say)
    if first.startswith("-"):
        raise CliError(f"unrecognized option '{first}'. For more information, try '--help'.")
    raise CliError(f"unrecognized command '{first}'. For more information, try '--help'.")


# ---- apply (main.rs:256-656) ----

# option -> (field, kind): kind "s" string, "f" float, "u" unsigned integer, None a switch.
_APPLY_OPTIONS = {
    "-o": ("output", "s"), "--output": ("output", "s"), "-p": ("preset", "s"), "--preset": ("preset", "s"),
    "-f": ("format", "s"), "--format": ("format", "s"), "--push": ("push", "f"), "--eberhard": ("eberhard", "f"),
    "--no-scanner-otf": ("no_otf", None), "-c": ("color", None), "--color": ("color", None), "--gpu": ("gpu", None),
    "-e": ("exposure", "f"), "--exposure": ("exposure", "f"), "-s": ("grain_size", "f"),
    "--grain-size": ("grain_size", "f"), "--grain-strength": ("grain_strength", "f"), "--scale": ("scale", "f"),
    "--auto-scale": ("auto_scale", None), "--reference-res": ("reference_res", "u"),
    "--supersample": ("supersample", "u"), "--tile-size": ("tile_size", "u"), "-w": ("width", "u"),
    "--width": ("width", "u"), "--height": ("height", "u"),
}


def _parse_value(opt: str, text: str, kind: str):
    if kind == "s":
        return text
    if kind == "f":
        try:
            return float(text)
        except ValueError:
            if opt == "--push":
                raise CliError(f"invalid value '{text}' for '--push': expected a positive number") from None
            raise CliError(f"invalid value '{text}' for '{opt}': expected a number") from None
    try:
        digits = text[1:] if text.startswith("+") else text
        if not digits.isdigit():
            raise ValueError
        v = int(digits)
        if v > 0xFFFFFFFF:
            raise ValueError
    except ValueError:
        hint = "an integer (1-4)" if opt == "--supersample" else "an integer"
        raise CliError(f"invalid value '{text}' for '{opt}': expected {hint}") from None
    return v


def parse_apply_args(args: list[str]) -> dict:
    """The option loop of main.rs:285-468; returns the raw settings (None where not given)."""
    s = {"input": None, "output": None, "preset": "tri-x", "format": None, "color": False, "exposure": 1.0,
         "grain_size": None, "grain_strength": None, "scale": 1.0, "auto_scale": False, "reference_res": 6000,
         "supersample": 1, "tile_size": 320, "width": None, "height": None, "gpu": False, "push": None,
         "eberhard": None, "no_otf": False}
    i = 0
    while i < len(args):
        a = args[i]
        if a in _APPLY_OPTIONS:
            field, kind = _APPLY_OPTIONS[a]
            if kind is None:
                s[field] = True
            else:
                i += 1
                if i >= len(args):
                    raise CliError(f"option '{a}' requires an argument")
                s[field] = _parse_value(a, args[i], kind)
        elif a.startswith("-"):
            raise CliError(f"unrecognized option '{a}'. For more information, try 'fgrain apply --help'.")
        elif s["input"] is None:
            s["input"] = a
        elif s["output"] is None:
            s["output"] = a
        else:
            raise CliError(f"unexpected positional argument '{a}'. For more information, try 'fgrain apply --help'.")
        i += 1
    if s["push"] is not None:
        s["push"] = max(s["push"], 0.0)
    if s["eberhard"] is not None:
        s["eberhard"] = max(s["eberhard"], 0.0)
    s["supersample"] = min(max(s["supersample"], 1), 4)
    return s


def apply_options(s: dict, say=print):
    """Defaults that depend on the stock and format (main.rs:478-540) and the render options."""
    from .film import FilmRenderOptions

    preset = s["preset"]
    low = preset.lower()
    push_preset = "1600" in low or low == "caffenol"
    push = s["push"] if s["push"] is not None else (2.0 if push_preset else 0.0)
    strength = s["grain_strength"] if s["grain_strength"] is not None else (1.25 if push_preset or push >= 1.5 else 1.0)
    eberhard = s["eberhard"] if s["eberhard"] is not None else 0.0
    fmt = (s["format"] or "35mm").lower()
    format_scale = 0.55 if fmt in ("120", "medium") else (0.28 if fmt in ("4x5", "large") else 1.0)
    if low in ("t-max", "tmax"):
        base = 1.1
    elif low in ("hp5", "hp5-plus"):
        base = 1.8
    elif low in ("tri-x-1600", "trix-1600", "caffenol"):
        base = 2.2
    else:
        base = 2.2 if push >= 1.5 else 2.4
    if s["grain_size"] is None:
        grain = base * format_scale
    elif s["grain_size"] < 0.05:
        say(f"[Notice] Grain size {s['grain_size']:.2f}px clamped to 0.05px minimum limit")
        grain = 0.05
    else:
        if s["grain_size"] > 4.5:
            say(f"[Notice] Grain size {s['grain_size']:.2f}px exceeds standard 35mm physical scale (~0.8-2.5px); "
                "rendering as extreme macro / sub-miniature crop")
        grain = s["grain_size"]
    w, h = s["width"], s["height"]
    out_dims = None if w is None and h is None else (w or 0, h or 0)
    return FilmRenderOptions(preset=preset, grain_size_px=grain, grain_strength=strength, exposure=s["exposure"],
                             color=s["color"], output_resolution=out_dims, tile_size=s["tile_size"], seed=42,
                             gpu=s["gpu"], auto_scale=s["auto_scale"], scale=s["scale"],
                             reference_res=s["reference_res"], supersample=s["supersample"], push=push,
                             eberhard=eberhard, scanner_otf=not s["no_otf"])


def safe_save(img: np.ndarray, path: str, say_err=None) -> str:
    """safe_save_gray / safe_save_rgb (image_pipeline.rs:1087-1133): when the file cannot be
    written, save beside it as <stem>_<unix seconds>.<ext> with a warning."""
    try:
        imageio.write_image(path, img)
        return path
    except imageio.ImageFormatError:
        raise
    except OSError as exc:
        p = Path(path)
        fallback = p.parent / f"{p.stem or 'output'}_{int(time.time())}{p.suffix or '.png'}"
        (say_err or (lambda m: print(m, file=sys.stderr)))(
            f"warning: file {str(p)!r} is locked ({exc}). Saving to fallback: {str(fallback)!r}")
        imageio.write_image(fallback, img)
        return str(fallback)


def run_image_apply(args: list[str], say=print) -> None:
    if not args or any(a in ("-h", "--help") for a in args):
        say(_APPLY_HELP)
        if not args:
            raise CliError("missing required argument <input_image>\n\nFor more information, try 'fgrain apply --help'.")
        return
    s = parse_apply_args(args)
    if s["input"] is None:
        raise CliError("missing required argument <input_image>\n\nUsage: fgrain apply <input_image> [output_image] "
                       "[options]\nFor more information, try 'fgrain apply --help'.")
    output = s["output"] or "film_grained_output.png"
    opts = apply_options(s, say)
    from .api import get_gpu_engine
    from .film import render_film

    say(f"[Input]  {s['input']}")
    say(f"[Output] {output}")
    say(f"[Preset] {opts.preset} ({'Color Multi-Layer' if opts.color else 'B&W Panchromatic'})")
    engine = get_gpu_engine()
    if engine is None:
        raise CliError("no CUDA device is available (this renderer has no CPU path)")
    say(f"[Acceleration] GPU ({engine.adapter_name()})")
    say(f"[Format] {s['format'] or '35mm'} | [Grain Size] {opts.grain_size_px:.2f}px | "
        f"[Grain Strength] {opts.grain_strength:.2f} | [Scale] {opts.scale:.2f}x")
    otf = "Active (Epson V850 MTF)" if opts.scanner_otf else "Disabled"
    if opts.push > 0.0:
        say(f"[Push Processing] +{opts.push:.1f} stops | [Eberhard Adjacency] {opts.eberhard:.2f}x | [Scanner OTF] {otf}")
    else:
        say(f"[Eberhard Adjacency] {opts.eberhard:.2f}x | [Scanner OTF] {otf}")
    if opts.auto_scale:
        say(f"[Auto-Scale] Active (relative to {opts.reference_res}px 35mm scan)")
    if opts.supersample > 1:
        say(f"[Supersampling] {opts.supersample}x optical scanner aperture integration")
    say(f"[Exposure Scale] {opts.exposure:.2f}x")
    say("\nProcessing image tiles...")
    try:
        img = imageio.read_image(s["input"])
        if opts.color and img.ndim == 2:
            img = np.repeat(img[:, :, None], 3, axis=2)  # to_rgb8 of a gray image
        rep, out = render_film(img, opts, engine)
        saved = safe_save(out, output)
    except (OSError, ValueError) as exc:  # ImageFormatError is a ValueError; GpuError a RuntimeError
        raise CliError(f"failed to process image '{s['input']}': {exc}") from None
    say("\nRender complete:")
    say(f"   Input Resolution:  {rep.input_resolution[0]}x{rep.input_resolution[1]}")
    say(f"   Output Resolution: {rep.output_resolution[0]}x{rep.output_resolution[1]}")
    say(f"   Total Tiles:       {rep.total_tiles}")
    say(f"   Total Crystals:    {rep.total_crystals}")
    say(f"   Developed Silver:  {rep.developed_crystals} "
        f"({rep.developed_crystals / max(rep.total_crystals, 1) * 100.0:.1f}%)")
    say(f"   Silver Clumps:     {rep.total_clumps}")
    say(f"   Processing Time:   {rep.elapsed_seconds:.2f}s")
    say(f"\nSaved output to: {saved}")


# ---- demonstrations (main.rs:659-1052) ----

def _run_demo_cli(name: str, args: list[str], say=print) -> None:
    if any(a in ("-h", "--help") for a in args):
        say(_demo_help(name))
        return
    output = None
    i = 0
    while i < len(args):
        a = args[i]
        if a in ("-o", "--output"):
            i += 1
            if i >= len(args):
                raise CliError(f"option '{a}' requires an argument")
            output = args[i]
        elif a.startswith("-"):
            raise CliError(f"unrecognized option '{a}' for '{name}'. For more information, try 'fgrain {name} --help'.")
        elif output is None:
            output = a
        else:
            raise CliError(f"unexpected positional argument '{a}'. For more information, try 'fgrain {name} --help'.")
        i += 1
    run_demo(name, output, say)


# Each demo: (preset, patch um, output px, synthesis seed, exposure cfg, exposure seed, exposure(x, y),
# scan seed).  The closure the reference passes to expose_emulsion is sampled on a DEMO_SAMPLE_UM
# grid and read back by the nearest-sample rule of the exposure-tile entry point.
DEMO_SAMPLE_UM = 0.1


def _demo_spec(name: str):
    from .api import ExposureConfig

    if name == "gradient":  # main.rs:800-895
        return ("tri-x", 60.0, 384, 42, ExposureConfig(6.0, 0.12, 1.3, 48), 1001,
                lambda x, y: 0.02 + 0.98 * np.clip(x / 60.0, 0.0, 1.0) ** 1.4, 2002)
    if name == "halation":  # main.rs:897-958
        return ("tri-x", 50.0, 256, 777, ExposureConfig(8.0, 0.15, 1.0, 64), 888,
                lambda x, y: np.where(np.hypot(x - 25.0, y - 25.0) < 4.0, 1.2, 0.04), 999)
    # tri-x, t-max: main.rs:960-1019
    return (name, 50.0, 256, 555, ExposureConfig(6.0, 0.12, 1.3, 48), 666, lambda x, y: np.full_like(x, 0.45), 777)


def demo_exposure_tile(fn, size_um: float) -> np.ndarray:
    """The closure sampled at the centres of a DEMO_SAMPLE_UM grid over the patch."""
    n = max(int(round(size_um / DEMO_SAMPLE_UM)), 2)
    c = (np.arange(n) + 0.5) * (size_um / n)
    x, y = np.meshgrid(c, c)
    return np.maximum(fn(x, y), 0.0).astype(np.float32)


def run_demo(name: str, output: str | None, say=print):
    from .api import (DevelopmentConfig, EmulsionConfig, ScanConfig, ScanMode, VirtualEmulsionLayer,
                      develop_emulsion, expose_emulsion, get_gpu_engine, scan_emulsion)

    preset, size, res, sseed, ecfg, eseed, fn, scseed = _demo_spec(name)
    engine = get_gpu_engine()
    if engine is None:
        raise CliError("no CUDA device is available (this renderer has no CPU path)")
    t0 = time.perf_counter()
    cfg = EmulsionConfig.t_max_100(size, size) if preset == "t-max" else EmulsionConfig.tri_x_400(size, size)
    say(f"\n[{name}] Synthesizing emulsion ({preset}, {size:.1f}x{size:.1f}x{cfg.dimensions[2]:.1f} um)...")
    em = VirtualEmulsionLayer.synthesize(cfg, sseed, engine)
    say(f"      Synthesized {len(em)} crystals")
    expose_emulsion(em, demo_exposure_tile(fn, size), ecfg, eseed)
    rep = develop_emulsion(em, DevelopmentConfig(4, 1.35, 1.25, 0.85))
    say(f"      Developed: {rep.developed_crystals} / {rep.total_crystals} crystals "
        f"({rep.developed_crystals / max(rep.total_crystals, 1) * 100.0:.1f}%)")
    say(f"      Clumps: {rep.total_clumps} | Max clump size: {rep.max_clump_size} grains | "
        f"Avg clump: {rep.avg_clump_size:.2f} grains")
    _, image = scan_emulsion(em, ScanConfig(res, res, 4, ScanMode.PositivePrint, 0.40), scseed)
    out = output or f"film_grain_{name}.png"
    try:
        imageio.write_image(out, image)
    except (OSError, ValueError) as exc:
        raise CliError(f"failed to save output image to '{out}': {exc}") from None
    say(f"\nRender complete. Saved output to: {out}")
    say(f"Total runtime: {time.perf_counter() - t0:.2f}s")


def main(argv=None) -> int:
    try:
        run_cli(list(sys.argv if argv is None else argv))
    except CliError as exc:
        print(f"error: {exc}", file=sys.stderr)
        return 1
    return 0
