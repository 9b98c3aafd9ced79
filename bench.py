#!/usr/bin/env python
"""Benchmark of the fgrain photon-transport and transmittance-scan path on GB300.

Headline workload (configuration C4, the largest that fits one GPU): a 4096 x 4096 RGB photograph
(per channel, uniform noise from seed 3 Gaussian-blurred with sigma 32 px, as 8-bit), t-max tabular
grains at 1.1 px, three dye layers, supersample 4 (16384^2 per layer), seed 42.  Its 8,112
overlapping tiles (52 x 52 per layer, up to 384 x 384 px) are rendered from exposure tile to
negative density by the batched graph path.  One step is one batch of 254 of those tiles (every
32nd tile of the photograph in layer-major grid order), so the step fits the timing budget; the
whole photograph is about 32 such batches.

Reported on one JSON line:
  value      output pixel-channels per second that the batch stands for (4096^2 x 3 x the batch's
             share of all tile pixels) over the device time per step, inputs resident in HBM.  The
             working set (crystals, trees, grids: tens of GB) is far larger than L2; no flush.
  e2e        the whole photograph through fg_render_film, host u8 pixels in, host u8 pixels out
             (luma split, upscale, PSF, every tile, blend and finish), one timed call.
  e2e_batch  the step's batch through the public batch API with page-locked host buffers: exposure
             tiles copied in and densities copied out every step.
  plain / batched_over_plain  the plain per-tile path (fg_render_tile: plan, copy, run, free per
             tile) against a batch of the same tiles, both host to host, on a 32-tile sample.
  roofline   the dominant kernel of the step against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a C++ restatement of the reference's Rayon CPU path with the
             reference's own hit rule) on 16 of the batch's tiles, one tile per host thread;
             mean_T_rel_err_vs_oracle compares those tiles' mean transmittance with the device's.
  c2, c3     the same quantities on configurations C2 and C3 (extra keys).

`--impl reference` times that CPU restatement alone (the reference itself is Rust and cannot be
built here; this arm imports nothing of the product) on C4 tiles from the same sample.  With
torchrun (N > 1) every rank renders its own replica (replicas only: no collective is involved).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpx/s and photons/s on 1 GB300, batched vs plain at <=0.5% mean-T error"
SEED = 42
M64 = 0xFFFFFFFFFFFFFFFF
COLOR_SEED_OFFSETS = (0, 10007, 20011)  # image_pipeline.rs:1048-1061

# C4
C4_SIDE = 4096
C4_SS = 4
C4_GRAIN = 1.1
C4_TILE = 320
C4_STRIDE = 32        # every 32nd tile of the photograph forms the step's batch
C4_PLAIN_EVERY = 8    # the plain-path sample: every 8th tile of the batch (32 tiles)
C4_CPU_EVERY = 16     # the CPU-oracle sample: every 16th tile of the batch (16 tiles)
C4_WORKLOAD = ("C4: 4096x4096 RGB blurred-noise photograph (sigma 32 px, seed 3, 8-bit), t-max tabular grains "
               "1.1 px, colour (three dye layers), supersample 4 (16384^2 per layer, 8112 tiles)")

# C2
C2_OUT = 1024
C2_SS = 2
C2_GRAIN = 2.4
C2_WORKLOAD = ("C2: 1024x1024 blurred-noise luminance (sigma 16, seed 1, gamma 2.2), tri-x, grain 2.4 px, push 0, "
               "supersample 2 (2048^2 internal, 49 tiles)")
C3_STOCKS = ("tri-x", "t-max", "hp5")


# ------------------------------------------------------------------------------------------------
# Inputs (synthetic: no dataset is involved)

def c4_image(side=C4_SIDE):
    """Per channel: uniform [0, 1) noise (numpy PCG64, seed 3, channels drawn in turn), Gaussian
    blur sigma 32 px (reflect), as 8-bit."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(3)
    planes = [np.clip(gaussian_filter(rng.random((side, side)), 32.0, mode="reflect"), 0.0, 1.0) for _ in range(3)]
    return np.ascontiguousarray(np.round(np.stack(planes, -1) * 255.0).astype(np.uint8))


def c4_sample(ntiles_per_layer, stride=C4_STRIDE):
    """(layer, tile index) of every `stride`-th tile of the photograph in layer-major grid order."""
    return [(k // ntiles_per_layer, k % ntiles_per_layer) for k in range(0, 3 * ntiles_per_layer, stride)]


def c2_inputs():
    from scipy.ndimage import gaussian_filter, zoom

    a = np.random.default_rng(1).random((C2_OUT, C2_OUT))
    lum = np.clip(gaussian_filter(a, 16.0, mode="reflect"), 0.0, None) ** 2.2
    return zoom(lum, C2_SS, order=1, mode="nearest").astype(np.float32)


def c2_tiles(exposure):
    import fgrain_gb300 as fg
    from fgrain_gb300.image import tile_grid, tile_seed

    H, W = exposure.shape
    grid, _, _ = tile_grid(W, H, C2_GRAIN)
    params = [fg.tile_params("tri-x", 1.0 / C2_GRAIN, t.tw, t.th, 1.0, 0.0, tile_seed(SEED, t)) for t in grid]
    tiles = [np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]) for t in grid]
    return grid, params, tiles


def c3_tiles():
    """Configuration C3: 64 square images, sides exp(U[ln 64, ln 512]) rounded, stock uniform over
    tri-x / t-max / hp5, push U[0, 3] stops, supersample uniform over 1-4 (master seed 0); image k
    is blurred uniform noise (seed k, sigma side / 32 px, gamma 2.2) zoomed by its supersample
    factor.  All tiles of all images form one batch.  Returns (params, tiles, output px)."""
    import fgrain_gb300 as fg
    from scipy.ndimage import gaussian_filter, zoom
    from fgrain_gb300.image import default_grain_px, effective_push, tile_grid, tile_seed

    rng = np.random.default_rng(0)
    params, tiles, out_px = [], [], 0
    for k in range(64):
        side = int(round(float(np.exp(rng.uniform(np.log(64.0), np.log(512.0))))))
        stock = C3_STOCKS[int(rng.integers(0, 3))]
        push = float(rng.uniform(0.0, 3.0))
        ss = int(rng.integers(1, 5))
        a = np.random.default_rng(k).random((side, side))
        lum = np.clip(gaussian_filter(a, max(side / 32.0, 2.0), mode="reflect"), 0.0, None) ** 2.2
        exposure = (zoom(lum, ss, order=1, mode="nearest") if ss > 1 else lum).astype(np.float32)
        grain = default_grain_px(stock, push)
        H, W = exposure.shape
        grid, _, _ = tile_grid(W, H, grain)
        for t in grid:
            params.append(fg.tile_params(stock, 1.0 / grain, t.tw, t.th, 1.0, effective_push(stock, push),
                                         tile_seed(k, t)))
            tiles.append(np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]))
        out_px += side * side
    return params, tiles, out_px


# ------------------------------------------------------------------------------------------------
# Measurement helpers

class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except OSError:
            pass
        finally:
            try:
                os.unlink(self.path)
            except OSError:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = max((num(r[2]) for r in rows if num(r[2]) is not None), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        loaded = sorted(sm)[len(sm) // 2:] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows), "power_w_max": max((num(r[3]) or 0 for r in rows), default=None)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch.distributed as td

    td.init_process_group("gloo")
    return td.get_rank(), td.get_world_size(), int(os.environ.get("LOCAL_RANK", "0")), td


def reduce_max(td, v):
    if td is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def barrier(td):
    if td is not None:
        td.barrier()


def measured_peak():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch of the benchmark's batch from a committed ncu summary, or None."""
    try:
        for line in (ROOT / "profiles" / name).read_text().splitlines():
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except (OSError, ValueError):
        pass
    return None


def rooflines(stats, workload_key):
    """The transport and Bridson kernels against the measured HBM bandwidth (algorithmic bytes:
    transport 4 B exposure per photon + 8 B count read-modify-write per hit + 116 B per crystal
    read once; Bridson 4 B read + 4 B written per synthesis cell)."""
    peak, kind = measured_peak()
    P, H, N = stats["photons"], stats["hits"], stats["crystals"]
    t_alg = 4.0 * P + 8.0 * H + 116.0 * N
    t_ach = t_alg / (stats["transport_ms"] / 1e3) / 1e9 if stats["transport_ms"] > 0 else 0.0
    b_alg = 8.0 * stats["cells"]
    b_ach = b_alg / (stats["bridson_ms"] / 1e3) / 1e9 if stats["bridson_ms"] > 0 else 0.0
    rt = {"bound": "hbm", "kernel": "k_transport", "achieved": t_ach, "peak": peak, "unit": "GB/s",
          "frac": t_ach / peak, "peak_source": kind, "traffic": profile_traffic(f"k_transport_{workload_key}.md"),
          "alg_bytes_per_launch": t_alg, "ms_per_launch": stats["transport_ms"]}
    rb = {"bound": "hbm", "kernel": "k_bridson", "achieved": b_ach, "peak": peak, "unit": "GB/s",
          "frac": b_ach / peak, "peak_source": kind, "traffic": profile_traffic(f"k_bridson_{workload_key}.md"),
          "alg_bytes_per_launch": b_alg, "ms_per_launch": stats["bridson_ms"],
          "note": "issue- and barrier-bound (shared-memory Bridson rounds), not memory-bound"}
    dominant = rb if stats["bridson_ms"] > stats["transport_ms"] else rt
    return dominant, {"k_bridson": rb, "k_transport": rt}


def mean_T(d):
    return float((10.0 ** (-(np.asarray(d, np.float64) - 0.05))).mean())


def host_to_host(fg, batch, tiles, steps):
    """Seconds per step of the batch API with page-locked host buffers: exposure in, density out."""
    pin_in = [fg.PinnedArray(t.shape) for t in tiles]
    pin_out = [fg.PinnedArray(t.shape) for t in tiles]
    for pi, t in zip(pin_in, tiles):
        pi.array[...] = t

    def step():
        batch.set_exposure([p.array for p in pin_in])
        batch.run()
        batch.wait()
        batch.density_into([p.array for p in pin_out])

    step()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    secs = (time.perf_counter() - t0) / steps
    for p in pin_in + pin_out:
        p.free()
    return secs, sum(t.nbytes for t in tiles)


def oracle_tiles(jobs, threads):
    """Renders (stock, pixel um, exposure tile, seed) jobs with the CPU oracle (the reference's hit
    rule), one tile per host thread as the reference's rayon tile map does (image_pipeline.rs:427).
    Returns (seconds, densities)."""
    from oracle import oracle as orc

    orc.lib()

    def one(j):
        stock, px, tile, seed = j
        return orc.render_tile(stock, px, tile, 1.0, 0.0, seed, orc.FAITHFUL, 1)[0]

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        dens = list(ex.map(one, jobs))
    return time.perf_counter() - t0, dens


# ------------------------------------------------------------------------------------------------
# C4 (headline)

def c4_batch_inputs(fg, film, im, img, engine):
    """Exposure tiles of the C4 sample from the renderer's own stages (per layer: the channel
    upscaled to the render size with Lanczos3, then the camera gate and gelatin PSF)."""
    side = img.shape[0]
    R = side * C4_SS
    grid, _, _ = im.tile_grid(R, R, C4_GRAIN, C4_TILE)
    nt = len(grid)
    sample = c4_sample(nt)
    params, tiles = [], []
    for c in range(3):
        src = film.resize_u8(np.ascontiguousarray(img[..., c]), R, R, film.LANCZOS3, engine)
        heff, _ = film.gelatin_psf(src, engine)
        del src
        for cc, i in sample:
            if cc != c:
                continue
            t = grid[i]
            params.append(fg.tile_params("t-max", 1.0 / C4_GRAIN, t.tw, t.th, 1.0, 0.0,
                                         im.tile_seed((SEED + COLOR_SEED_OFFSETS[c]) & M64, t)))
            tiles.append(np.ascontiguousarray(heff[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]))
        del heff
    all_px = 3 * sum(t.tw * t.th for t in grid)
    return params, tiles, all_px, len(grid)


def run_c4(args):
    import fgrain_gb300 as fg
    from fgrain_gb300 import film
    from fgrain_gb300 import image as im

    rank, world, local, td = dist()
    side = args.film_side
    img = c4_image(side)
    out_pxc = side * side * 3
    engine = fg.GpuEngine(local)
    params, tiles, all_px, nt = c4_batch_inputs(fg, film, im, img, engine)
    sample_px = sum(p.width_px * p.height_px for p in params)
    rep_pxc = out_pxc * sample_px / all_px  # output pixel-channels the batch stands for

    batch = fg.Batch(params, engine, use_graph=True, autotune=True)
    batch.set_exposure(tiles)
    for _ in range(max(args.warmup, 0)):
        batch.run()
        batch.wait()
    barrier(td)
    with Clocks(local) as clk:
        ms = batch.time(args.steps)
    stats = batch.wait()
    barrier(td)
    clocks = clk.summary()
    per_step = reduce_max(td, ms) / args.steps
    value = world * rep_pxc / (per_step / 1e3) / 1e6
    d_batched = batch.density()
    e2e_steps = max(3, args.steps // 4)
    e2e_s, e2e_bytes = host_to_host(fg, batch, tiles, e2e_steps)
    e2e_s = reduce_max(td, e2e_s)
    batch.close()

    # Plain per-tile path against a batch of the same tiles, both host to host.
    sub = list(range(0, len(params), C4_PLAIN_EVERY))
    sp = [params[i] for i in sub]
    st_ = [tiles[i] for i in sub]
    fg.render_tile(st_[0], sp[0], engine)  # warm-up
    t0 = time.perf_counter()
    d_plain = [fg.render_tile(t, p, engine) for t, p in zip(st_, sp)]
    plain_s = time.perf_counter() - t0
    sub_pxc = out_pxc * sum(p.width_px * p.height_px for p in sp) / all_px
    b2 = fg.Batch(sp, engine, use_graph=True, autotune=True)
    b2_s, _ = host_to_host(fg, b2, st_, 3)
    b2.close()
    plain_identical = all(np.array_equal(d_batched[i], d) for i, d in zip(sub, d_plain))

    dominant, rls = rooflines(stats, "c4")
    res = {}
    if rank == 0 and world == 1 and not args.no_cpu:
        # CPU oracle on 16 tiles of the batch, one tile per thread; mean T against the device's.
        threads = min(os.cpu_count() or 1, 16)
        csub = list(range(0, len(params), C4_CPU_EVERY))[:16]
        jobs = [("t-max", 1.0 / C4_GRAIN, tiles[i], params[i].seed) for i in csub]
        secs, dens = oracle_tiles(jobs, threads)
        cpu_pxc = out_pxc * sum(params[i].width_px * params[i].height_px for i in csub) / all_px
        res["cpu_baseline"] = {
            "value": cpu_pxc / secs / 1e6, "unit": "Mpx/s", "cores": threads, "kind": "port",
            "sample": f"{len(csub)} of the C4 batch's tiles (every {C4_STRIDE * C4_CPU_EVERY}th tile of the photograph), "
                      f"one tile per thread on {threads} threads, C++ restatement of the reference CPU path with the "
                      f"reference's hit rule; output pixel-channels scaled by tile pixels"}
        Td = np.array([mean_T(d_batched[i]) for i in csub])
        To = np.array([mean_T(d) for d in dens])
        res["mean_T_rel_err_vs_oracle"] = float(abs(Td.mean() - To.mean()) / To.mean())
        res["mean_T_vs_oracle"] = {"device": float(Td.mean()), "oracle": float(To.mean()), "tiles": len(csub),
                                   "per_tile_rel_sd": float(np.std(To) / To.mean())}

    # The whole photograph through fg_render_film, host pixels to host pixels.
    opts = film.FilmRenderOptions(preset="t-max", grain_size_px=C4_GRAIN, supersample=C4_SS, color=True, seed=SEED,
                                  eberhard=0.5, batch_bytes=int(args.batch_gb * 2**30))
    film.render_film(img[:512, :512], opts, engine)  # warm-up on a corner
    barrier(td)
    t0 = time.perf_counter()
    rep, out = film.render_film(img, opts, engine)
    film_s = reduce_max(td, time.perf_counter() - t0)

    extras = {}
    if not args.no_extras:
        extras["c2"] = c2_extra(fg, engine, min(args.steps, 10))
        extras["c3"] = c3_extra(fg, engine, min(args.steps, 3))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": C4_WORKLOAD + (" (reduced size)" if side != C4_SIDE else "") +
                       f"; one step = one batch of {len(params)} of its {3 * nt} tiles (every {C4_STRIDE}th), "
                       "device-resident, batched graph path",
                       "tiles_per_step": len(params), "tiles_total": 3 * nt,
                       "output_px_channels_per_step": rep_pxc, "output_px_channels_total": out_pxc,
                       "l2": "working set (crystals, trees, grids) exceeds L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "photons_per_s": stats["photons"] / (stats["transport_ms"] / 1e3),
            "stage_ms": {k: stats[k] for k in ("synth_ms", "bridson_ms", "bvh_ms", "transport_ms", "develop_ms",
                                               "scan_ms", "total_ms")},
            "work": {k: stats[k] for k in ("crystals", "photons", "hits", "rays", "scan_hits", "scan_fallbacks",
                                           "cells", "developed", "clumps")},
            "launch_shape": {"transport_threads": stats["transport_threads"],
                             "transport_blocks": stats["transport_blocks"], "scan_bin_px": stats["scan_bin_px"]},
            "e2e": {"value": out_pxc * world / film_s / 1e6, "unit": "Mpx/s", "h2d_bytes_per_step": int(img.nbytes),
                    "d2h_bytes_per_step": int(out.nbytes), "steps": 1,
                    "what": "the whole photograph per fg_render_film call, host u8 pixels to host u8 pixels",
                    "seconds": film_s, "tiles": rep.total_tiles, "crystals": rep.total_crystals,
                    "photons": rep.photons, "stage_ms": rep.extra},
            "e2e_batch": {"value": world * rep_pxc / e2e_s / 1e6, "unit": "Mpx/s", "h2d_bytes_per_step": e2e_bytes,
                          "d2h_bytes_per_step": e2e_bytes, "steps": e2e_steps,
                          "what": "the step's batch through the batch API, page-locked host buffers"},
            "plain_mpx_s": sub_pxc / plain_s / 1e6,
            "batched_host_mpx_s": sub_pxc / b2_s / 1e6,
            "batched_over_plain": plain_s / b2_s,
            "batched_over_plain_basis": f"{len(sp)} tiles of the batch, both host to host: fg_render_tile per tile "
                                        "against one batch of the same tiles (exposure in, density out)",
            "batched_equals_plain_bitwise": plain_identical,
            "gpu_launches": stats["kernel_launches"] * args.steps,
            "roofline": dominant,
            "rooflines": rls,
            "clocks": clocks,
        }
        line.update(res)
        line.update(extras)
        print(json.dumps(line))
    if td:
        td.destroy_process_group()


def c2_extra(fg, engine, steps):
    exposure = c2_inputs()
    grid, params, tiles = c2_tiles(exposure)
    b = fg.Batch(params, engine, use_graph=True, autotune=True)
    b.set_exposure(tiles)
    for _ in range(2):
        b.run()
        b.wait()
    ms = b.time(steps) / steps
    stats = b.wait()
    d_b = b.density()
    h_s, h_bytes = host_to_host(fg, b, tiles, 3)
    b.close()
    t0 = time.perf_counter()
    d_p = [fg.render_tile(t, p, engine) for t, p in zip(tiles, params)]
    plain_s = time.perf_counter() - t0
    px = C2_OUT * C2_OUT
    dominant, _ = rooflines(stats, "c2")
    return {"workload": C2_WORKLOAD, "value": px / (ms / 1e3) / 1e6, "ms_per_step": ms, "steps": steps,
            "e2e_batch": {"value": px / h_s / 1e6, "h2d_bytes_per_step": h_bytes, "d2h_bytes_per_step": h_bytes},
            "plain_mpx_s": px / plain_s / 1e6, "batched_over_plain": plain_s / h_s,
            "batched_over_plain_device": plain_s / (ms / 1e3),
            "batched_equals_plain_bitwise": all(np.array_equal(x, y) for x, y in zip(d_b, d_p)),
            "photons_per_s": stats["photons"] / (stats["transport_ms"] / 1e3),
            "stage_ms": {k: stats[k] for k in ("synth_ms", "bridson_ms", "bvh_ms", "transport_ms", "develop_ms",
                                               "scan_ms", "total_ms")},
            "roofline": dominant}


def c3_extra(fg, engine, steps):
    params, tiles, out_px = c3_tiles()
    b = fg.Batch(params, engine, use_graph=True, autotune=True)
    b.set_exposure(tiles)
    b.run()
    b.wait()
    ms = b.time(steps) / steps
    stats = b.wait()
    d_b = b.density()
    h_s, h_bytes = host_to_host(fg, b, tiles, 1)
    b.close()
    t0 = time.perf_counter()
    d_p = [fg.render_tile(t, p, engine) for t, p in zip(tiles, params)]
    plain_s = time.perf_counter() - t0
    return {"workload": "C3: 64 square images, sides log-uniform 64-512 px, tri-x / t-max / hp5, push 0-3, "
                        "supersample 1-4 (master seed 0), all tiles in one autotuned batch",
            "tiles": len(params), "value": out_px / (ms / 1e3) / 1e6, "ms_per_step": ms, "steps": steps,
            "e2e_batch": {"value": out_px / h_s / 1e6, "h2d_bytes_per_step": h_bytes, "d2h_bytes_per_step": h_bytes},
            "plain_mpx_s": out_px / plain_s / 1e6, "batched_over_plain": plain_s / h_s,
            "batched_over_plain_device": plain_s / (ms / 1e3),
            "batched_equals_plain_bitwise": all(np.array_equal(x, y) for x, y in zip(d_b, d_p)),
            "stage_ms": {k: stats[k] for k in ("synth_ms", "bridson_ms", "bvh_ms", "transport_ms", "develop_ms",
                                               "scan_ms", "total_ms")}}


# ------------------------------------------------------------------------------------------------
# C2 / C3 / fast as lines of their own (not the headline)

def run_single(args):
    import fgrain_gb300 as fg

    rank, world, local, td = dist()
    engine = fg.GpuEngine(local)
    d = c2_extra(fg, engine, args.steps) if args.workload == "c2" else c3_extra(fg, engine, args.steps)
    if rank == 0:
        px_step = d["value"] * d["ms_per_step"] / 1e3
        print(json.dumps({
            "metric": METRIC, "value": d["value"] * world, "unit": "Mpx/s", "n_gpus": world, "steps": d["steps"],
            "warmup": 2 if args.workload == "c2" else 1, "ms_per_step": d["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": d["workload"], "output_px_per_step": px_step, "parallelism": f"replicas x{world}"},
            "e2e": {"value": d["e2e_batch"]["value"], "unit": "Mpx/s",
                    "h2d_bytes_per_step": d["e2e_batch"]["h2d_bytes_per_step"],
                    "d2h_bytes_per_step": d["e2e_batch"]["d2h_bytes_per_step"]},
            "details": d}))


def run_fast(args):
    """The C2 tiles through the fast-approximation mode (the reference's wgpu tile model, with the
    GPU branch's tile parameters): one fg_render_tiles_fast call per step, host tiles in and host
    densities out.  Reported next to the headline, not instead of it."""
    import fgrain_gb300 as fg
    from fgrain_gb300 import fast
    from fgrain_gb300.image import tile_grid, tile_seed

    rank, world, local, td = dist()
    exposure = c2_inputs()
    H, W = exposure.shape
    grid, _, _ = tile_grid(W, H, C2_GRAIN)
    params = [fast.tile_params_fast("tri-x", 1.0 / C2_GRAIN, t.tw, t.th, 1.0, 0.0, tile_seed(SEED, t)) for t in grid]
    tiles = [np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]) for t in grid]
    engine = fg.GpuEngine(local)
    for _ in range(max(args.warmup, 0)):
        fast.render_tiles_fast(params, tiles, engine)
    barrier(td)
    with Clocks(local) as ck:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fast.render_tiles_fast(params, tiles, engine)
        t = (time.perf_counter() - t0) / args.steps
    t = reduce_max(td, t)
    if rank == 0:
        value = C2_OUT * C2_OUT * world / t / 1e6
        h2d = sum(x.nbytes for x in tiles)
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "C2 tiles through the fast approximation (the reference's wgpu tile model: "
                                   "jittered grid, per-crystal Poisson counts, column scan), host to host",
                       "tiles": len(grid), "output_px": C2_OUT * C2_OUT, "parallelism": f"replicas x{world}"},
            "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
            "gpu_launches": 5 * args.steps, "clocks": ck.summary()}))


# ------------------------------------------------------------------------------------------------
# Reference arm: the CPU restatement of the reference path, oracle only

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as orc

    side = args.film_side
    img = c4_image(side)
    out_pxc = side * side * 3
    R = side * C4_SS
    grid, _, _ = orc.film_grid(R, R, C4_GRAIN, C4_TILE)
    nt = len(grid)
    sample = c4_sample(nt)
    threads = os.cpu_count() or 1
    # 4 tiles per step, rounded up to whole waves of the thread pool: the reference's rayon tile map
    # over a photograph's thousands of tiles keeps every core busy.
    warm_n = max(args.warmup, 0)
    timed_n = -(-4 * args.steps // threads) * threads
    picks = [sample[k % len(sample)] for k in range(warm_n + timed_n)]
    heffs = {}
    for c in sorted({c for c, _ in picks}):  # the oracle's own exposure stages (upscale, PSF)
        src = orc.resize_u8(np.ascontiguousarray(img[..., c]), R, R, orc.LANCZOS3)
        heffs[c] = orc.gelatin_psf(src)[0]
        del src
    jobs = []
    for c, i in picks:
        t = grid[i]
        jobs.append(("t-max", 1.0 / C4_GRAIN,
                     np.ascontiguousarray(heffs[c][t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]),
                     orc.film_tile_seed((SEED + COLOR_SEED_OFFSETS[c]) & M64, t)))
    heffs.clear()
    if warm_n:
        oracle_tiles(jobs[:warm_n], threads)
    secs, _ = oracle_tiles(jobs[warm_n:], threads)
    all_px = 3 * sum(t.tw * t.th for t in grid)
    px = sum(j[2].size for j in jobs[warm_n:])
    value = out_pxc * px / all_px / secs / 1e6
    sample_txt = (f"{timed_n} C4 tiles for {args.steps} steps (the first of the benchmark's every-{C4_STRIDE}th-tile "
                  f"sample, 4 per step rounded up to whole waves of the {threads}-thread tile map, rendered together as "
                  f"the reference's rayon map renders tiles); C++ restatement of the reference CPU path with the reference's hit rule (the Rust "
                  f"reference cannot be built here); output pixel-channels scaled by tile pixels; each warm-up step "
                  f"renders one tile")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": C4_WORKLOAD + ", reference CPU path (no GPU used)", "tiles_per_step": timed_n / args.steps},
        "cpu_baseline": {"value": value, "unit": "Mpx/s", "cores": threads, "kind": "port", "sample": sample_txt},
        "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_profile(args):
    """One batched run of the workload's batch between cudaProfilerStart and cudaProfilerStop, for
    `ncu --profile-from-start off`: c2, its 49 tiles; c4, the first --profile-region tiles of the C4
    step's batch.  Warm-up runs (autotune, graph capture) come first and are not profiled."""
    import torch.cuda.profiler as prof
    import fgrain_gb300 as fg

    engine = fg.GpuEngine(0)
    if args.workload == "c2":
        exposure = c2_inputs()
        _, params, tiles = c2_tiles(exposure)
    else:
        from fgrain_gb300 import film
        from fgrain_gb300 import image as im

        params, tiles, _, _ = c4_batch_inputs(fg, film, im, c4_image(args.film_side), engine)
        params, tiles = params[:args.profile_region], tiles[:args.profile_region]
    batch = fg.Batch(params, engine, use_graph=True, autotune=True)
    batch.set_exposure(tiles)
    for _ in range(max(args.warmup, 1)):
        batch.run()
        batch.wait()
    prof.start()
    batch.run()
    st = batch.wait()
    prof.stop()
    batch.close()
    print(json.dumps({"profile_region": args.workload, "tiles": len(params),
                      **{k: st[k] for k in ("synth_ms", "bvh_ms", "transport_ms", "develop_ms", "scan_ms", "total_ms",
                                            "kernel_launches", "crystals", "photons", "hits")}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed steps")
    ap.add_argument("--warmup", type=int, default=3, help="untimed steps")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true", help="skip the C2 and C3 keys of the C4 line")
    ap.add_argument("--workload", choices=["c4", "c2", "c3", "fast"], default="c4",
                    help="c4: the headline (C4 with C2 and C3 as extra keys); c2, c3: those configurations alone; "
                         "fast: the C2 tiles through the fast approximation")
    ap.add_argument("--film-side", type=int, default=C4_SIDE, help="side of the C4 photograph (4096 for C4)")
    ap.add_argument("--batch-gb", type=float, default=0.0,
                    help="device GiB one batch of the whole-photograph render may use (0: 70 %% of the free memory)")
    ap.add_argument("--profile-region", type=int, default=0, metavar="TILES",
                    help="run one batch between cudaProfilerStart/Stop and exit (ncu --profile-from-start off): "
                         "c2, its 49 tiles; c4, the first TILES tiles of the C4 step's batch")
    args = ap.parse_args()
    if args.profile_region:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.workload == "fast":
        run_fast(args)
    else:
        run_single(args)


if __name__ == "__main__":
    main()
