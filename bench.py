#!/usr/bin/env python
"""Benchmark of the fgrain photon-transport and transmittance-scan path on GB300.

Workload (one "step"): the 1024 x 1024 black-and-white image of configuration C2 rendered at
supersample 2 (2048 x 2048 internal, tri-x cubic grains, grain 2.4 px, push 0, seed 42): 49
overlapping tiles of up to 384 x 384 px, each synthesized, exposed, developed and scanned to
negative density by the batched graph path.  Inputs: blurred uniform noise (sigma 16 px, seed 1,
gamma 2.2) upsampled x2 by linear interpolation (synthetic; no dataset is involved).

Reported:
  value      output Mpx/s (1024^2 output pixels per step / device time per step), inputs resident
             in HBM; the working set (crystals, LBVH, grids) is several GB, far larger than L2.
  e2e        the same through the public API with page-locked host buffers: host->device copy of
             the exposure tiles, run, device->host copy of the density tiles, every step.
  roofline   the transport kernel against the measured HBM copy bandwidth.
  cpu_baseline  the CPU oracle (a C++ restatement of the reference's Rayon CPU path, faithful
             hit rule) on a bounded sample of the same tiles, all host threads.

`--impl reference` times that CPU restatement alone (the reference itself is Rust and cannot be
built here) on the same workload, metric and unit.  With torchrun (N > 1) every rank renders its
own replica of the image (replicas only: no collective is involved), and rank 0 reports the sum.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpx/s and photons/s on 1 GB300, batched vs plain at <=0.5% mean-T error"
OUT_W = OUT_H = 1024
SS = 2
GRAIN = 2.4
SEED = 42


def c2_inputs():
    from scipy.ndimage import gaussian_filter, zoom

    a = np.random.default_rng(1).random((OUT_H, OUT_W))
    lum = np.clip(gaussian_filter(a, 16.0, mode="reflect"), 0.0, None) ** 2.2
    exposure = zoom(lum, SS, order=1, mode="nearest").astype(np.float32)
    return exposure


def c2_tiles(exposure, ntiles=None):
    import fgrain_gb300 as fg
    from fgrain_gb300.image import tile_grid, tile_seed

    H, W = exposure.shape
    grid, step, pad = tile_grid(W, H, GRAIN)
    if ntiles:
        grid = grid[:ntiles]
    params, tiles = [], []
    for t in grid:
        params.append(fg.tile_params("tri-x", 1.0 / GRAIN, t.tw, t.th, 1.0, 0.0, tile_seed(SEED, t)))
        tiles.append(np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]))
    return grid, params, tiles


C3_STOCKS = ("tri-x", "t-max", "hp5")


def c3_tiles():
    """Configuration C3: 64 square images, sides exp(U[ln 64, ln 512]) rounded, stock uniform over
    tri-x / t-max / hp5, push U[0, 3] stops, supersample uniform over 1-4 (master seed 0); image k
    is blurred uniform noise (seed k, sigma side / 32 px, gamma 2.2) zoomed by its supersample
    factor.  All tiles of all images form one batch.  Returns (params, tiles, output px, internal
    px)."""
    import fgrain_gb300 as fg
    from scipy.ndimage import gaussian_filter, zoom
    from fgrain_gb300.image import default_grain_px, effective_push, tile_grid, tile_seed

    rng = np.random.default_rng(0)
    params, tiles, out_px, int_px = [], [], 0, 0
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
        int_px += W * H
    return params, tiles, out_px, int_px


def c2_tiles_grid(exposure):
    from fgrain_gb300.image import tile_grid

    return tile_grid(exposure.shape[1], exposure.shape[0], GRAIN)[0]


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


def oracle_sample(params, tiles, ntiles, threads):
    """Renders `ntiles` tiles with the CPU oracle (faithful hit rule), tiles in parallel the way the
    reference's rayon map does (image_pipeline.rs:427); returns (seconds, tile pixels)."""
    from oracle import oracle as orc

    idx = list(range(min(ntiles, len(params))))

    def one(i):
        p = params[i]
        orc.render_tile("tri-x", 1.0 / GRAIN, tiles[i], p.exposure, 0.0, p.seed, orc.FAITHFUL, 1)
        return p.width_px * p.height_px

    orc.lib()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        px = sum(ex.map(one, idx))
    return time.perf_counter() - t0, px


def measured_peak():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(name="k_transport_c2.md"):
    """dram bytes per launch of the full C2 workload from a committed ncu summary, or None."""
    f = ROOT / "profiles" / name
    try:
        for line in f.read_text().splitlines():
            if line.strip().startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except (OSError, ValueError):
        pass
    return None


def run_ours(args):
    import fgrain_gb300 as fg

    rank, world, local, td = dist()
    if args.workload == "c3":
        params, tiles, c3_out_px, c3_int_px = c3_tiles()
        exposure = None
    else:
        exposure = c2_inputs()
        grid, params, tiles = c2_tiles(exposure, args.tiles)
    engine = fg.GpuEngine(local)
    batch = fg.Batch(params, engine, use_graph=True, autotune=True)
    batch.set_exposure(tiles)
    for _ in range(max(args.warmup, 0)):
        batch.run()
        stats = batch.wait()
    batch.run()
    stats = batch.wait()
    d_batched = batch.density()
    if td:
        td.barrier()
    prof = None
    if args.profile_region:  # limits an `ncu --profile-from-start off` capture to the timed replays
        import torch.cuda.profiler as prof
        prof.start()
    with Clocks(local) as clk:
        ms = batch.time(args.steps)
    if prof:
        prof.stop()
    stats = batch.wait()  # stage times of the last timed replay (CUDA events on the engine stream)
    if td:
        td.barrier()
    clocks = clk.summary()
    ms_max = reduce_max(td, ms)
    per_step = ms_max / args.steps
    full = not args.tiles or args.tiles >= 49
    if args.workload == "c3":
        out_px = c3_out_px
    else:
        out_px = OUT_W * OUT_H if full else int(round(OUT_W * OUT_H * sum(p.width_px * p.height_px for p in params)
                                                      / sum(t.tw * t.th for t in c2_tiles_grid(exposure))))
    value = world * out_px / (per_step / 1e3) / 1e6

    # End to end through the public API: pinned host exposure in, pinned density out, per step.
    pin_in = [fg.PinnedArray(t.shape) for t in tiles]
    pin_out = [fg.PinnedArray(t.shape) for t in tiles]
    for pi, t in zip(pin_in, tiles):
        pi.array[...] = t
    def e2e_step():
        batch.set_exposure([p.array for p in pin_in])
        batch.run()
        batch.wait()
        ptrs = [p.array for p in pin_out]
        import ctypes as C
        arr = (C.POINTER(C.c_float) * len(ptrs))(*[a.ctypes.data_as(C.POINTER(C.c_float)) for a in ptrs])
        st = engine._lib.fg_batch_get_density(batch._h, arr)
        if st != 0:
            raise RuntimeError("density copy failed")
    e2e_step()
    if td:
        td.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = reduce_max(td, time.perf_counter() - t0) / args.steps
    h2d = sum(t.nbytes for t in tiles)
    d2h = h2d
    e2e_value = world * out_px / e2e_s / 1e6

    # Plain per-tile path (one render_tile call per tile, each making and freeing its buffers).
    t0 = time.perf_counter()
    d_plain = [fg.render_tile(t, p, engine) for t, p in zip(tiles, params)]
    plain_s = time.perf_counter() - t0
    plain_value = out_px / plain_s / 1e6
    Tb = np.concatenate([(10.0 ** -(d.astype(np.float64) - 0.05)).ravel() for d in d_batched])
    Tp = np.concatenate([(10.0 ** -(d.astype(np.float64) - 0.05)).ravel() for d in d_plain])
    mean_t_err = abs(Tb.mean() - Tp.mean()) / Tp.mean()
    bit_identical = all(np.array_equal(a, b) for a, b in zip(d_batched, d_plain))

    # Roofline of the transport kernel: algorithmic bytes per launch = 4 B exposure gather per
    # photon + 8 B count read-modify-write per hit + 116 B per crystal (48 B record, 64 B node,
    # 4 B count zero) read once.
    P, H, N = stats["photons"], stats["hits"], stats["crystals"]
    alg_bytes = 4.0 * P + 8.0 * H + 116.0 * N
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (stats["transport_ms"] / 1e3) / 1e9
    photons_per_s = P / (stats["transport_ms"] / 1e3)
    c2_full = args.workload == "c2" and full
    rl_transport = {"bound": "hbm", "kernel": "k_transport", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "peak_source": peak_kind,
                    "traffic": profile_traffic() if c2_full else None, "alg_bytes_per_launch": alg_bytes,
                    "ms_per_launch": stats["transport_ms"]}
    # Roofline of the Bridson kernel: it stages every synthesis cell of its column and halo from the
    # tile's cell grid and writes the column back, so 4 B read + 4 B written per cell at least.
    b_alg = 8.0 * stats["cells"]
    b_ach = b_alg / (stats["bridson_ms"] / 1e3) / 1e9
    rl_bridson = {"bound": "hbm", "kernel": "k_bridson", "achieved": b_ach, "peak": peak, "unit": "GB/s",
                  "frac": b_ach / peak, "peak_source": peak_kind,
                  "traffic": profile_traffic("k_bridson_c2.md") if c2_full else None, "alg_bytes_per_launch": b_alg,
                  "ms_per_launch": stats["bridson_ms"],
                  "note": "issue- and barrier-bound (shared-memory Bridson rounds), not memory-bound"}
    dominant = rl_bridson if stats["bridson_ms"] > stats["transport_ms"] else rl_transport

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and args.workload == "c2":
        threads = os.cpu_count() or 1
        secs, px = oracle_sample(params, tiles, max(threads, 4), threads)
        total_px = sum(p.width_px * p.height_px for p in params)
        cpu_value = out_px * (px / total_px) / secs / 1e6
        cpu = {"value": cpu_value, "unit": "Mpx/s", "cores": threads, "kind": "port",
               "sample": f"{max(threads, 4)} of the 49 C2 tiles rendered by the C++ restatement of the "
                         f"reference CPU path (faithful hit rule), tiles in parallel; scaled by tile pixels"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": (("" if full else f"first {len(params)} tiles of ") + C2_WORKLOAD +
                                    ", batched graph path") if args.workload == "c2" else
                                   "C3: 64 square images, sides log-uniform 64-512 px, tri-x / t-max / hp5, push "
                                   "0-3, supersample 1-4 (master seed 0), all tiles in one autotuned batch",
                       "tiles": len(params),
                       "internal_px": int(exposure.size) if exposure is not None else int(c3_int_px),
                       "output_px": out_px, "l2": "working set (crystals, LBVH, grids) exceeds L2; no flush",
                       "parallelism": f"replicas x{world}"},
            "photons_per_s": photons_per_s,
            "plain_mpx_s": plain_value,
            "batched_over_plain": value / world / plain_value,
            "mean_T_rel_err_batched_vs_plain": mean_t_err,
            "batched_equals_plain_bitwise": bit_identical,
            "stage_ms": {k: stats[k] for k in ("synth_ms", "bridson_ms", "bvh_ms", "transport_ms", "develop_ms",
                                               "scan_ms", "total_ms")},
            "work": {k: stats[k] for k in ("crystals", "photons", "hits", "rays", "scan_hits", "scan_fallbacks",
                                           "cells", "developed", "clumps")},
            "launch_shape": {"transport_threads": stats["transport_threads"],
                             "transport_blocks": stats["transport_blocks"], "scan_bin_px": stats["scan_bin_px"]},
            "e2e": {"value": e2e_value, "unit": "Mpx/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": stats["kernel_launches"] * args.steps,
            "roofline": dominant,
            "rooflines": {"k_bridson": rl_bridson, "k_transport": rl_transport},
            "clocks": clocks,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    for p in pin_in + pin_out:
        p.free()
    batch.close()
    if td:
        td.destroy_process_group()


def run_c4(args):
    """C4: a 4096 x 4096 RGB photograph (three dye layers), t-max, grain 1.1 px, supersample 4, so
    16384^2 per channel and 2704 tiles per channel, rendered whole by fg_render_film from host
    pixels to host pixels (image stages, tiles in consecutive batches within the device budget,
    finish).  Inputs: per channel, blurred uniform noise (sigma 16 px) to the power 2.2, as u8.
    Reported next to the headline, not instead of it: value and e2e are the same host-to-host
    number, output pixel-channels per second."""
    import fgrain_gb300 as fg
    from fgrain_gb300 import film
    from scipy.ndimage import gaussian_filter

    rank, world, local, td = dist()
    rng = np.random.default_rng(1)
    side = args.film_side
    img = np.stack([np.clip(gaussian_filter(rng.random((side, side)), 16.0, mode="reflect"), 0.0, 1.0) ** 2.2
                    for _ in range(3)], -1)
    img = np.ascontiguousarray(np.round(img * 255.0).astype(np.uint8))
    opts = film.FilmRenderOptions(preset="t-max", grain_size_px=1.1, supersample=4, color=True, seed=SEED,
                                  batch_bytes=int(args.batch_gb * 2**30))
    engine = fg.GpuEngine(local)
    for _ in range(max(args.warmup, 0)):
        film.render_film(img, opts, engine)
    if td:
        td.barrier()
    times, reps = [], []
    with Clocks(local) as ck:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            rep, out = film.render_film(img, opts, engine)
            times.append(time.perf_counter() - t0)
            reps.append(rep)
    t = reduce_max(td, sum(times) / len(times))
    px = side * side * 3
    if rank == 0:
        value = px * world / t / 1e6
        rep = reps[-1]
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": (f"C4: {side}x{side} RGB blurred-noise photograph, t-max, grain 1.1 px, supersample 4 "
                                    f"({4 * side}^2 per channel), colour, whole photograph per fg_render_film call"
                                    + ("" if side == 4096 else " (reduced size)")),
                       "tiles": rep.total_tiles, "output_px_channels": px, "crystals": rep.total_crystals,
                       "photons": rep.photons, "parallelism": f"replicas x{world}",
                       "stage_ms": rep.extra},
            "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": img.nbytes, "d2h_bytes_per_step": out.nbytes},
            "clocks": ck.summary()}))


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
    grid, _, _ = tile_grid(W, H, GRAIN)
    params = [fast.tile_params_fast("tri-x", 1.0 / GRAIN, t.tw, t.th, 1.0, 0.0, tile_seed(SEED, t)) for t in grid]
    tiles = [np.ascontiguousarray(exposure[t.y_start:t.y_start + t.th, t.x_start:t.x_start + t.tw]) for t in grid]
    engine = fg.GpuEngine(local)
    for _ in range(max(args.warmup, 0)):
        fast.render_tiles_fast(params, tiles, engine)
    if td:
        td.barrier()
    with Clocks(local) as ck:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fast.render_tiles_fast(params, tiles, engine)
        t = (time.perf_counter() - t0) / args.steps
    t = reduce_max(td, t)
    if rank == 0:
        value = OUT_W * OUT_H * world / t / 1e6
        h2d = sum(x.nbytes for x in tiles)
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "C2 tiles through the fast approximation (the reference's wgpu tile model: "
                                   "jittered grid, per-crystal Poisson counts, column scan), host to host",
                       "tiles": len(grid), "output_px": OUT_W * OUT_H, "parallelism": f"replicas x{world}"},
            "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
            "gpu_launches": 5 * args.steps, "clocks": ck.summary()}))


C2_WORKLOAD = ("C2: 1024x1024 blurred-noise luminance (sigma 16, seed 1, gamma 2.2), tri-x, grain 2.4 px, push 0, "
               "supersample 2 (2048^2 internal, 49 tiles)")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    exposure = c2_inputs()
    grid, params, tiles = c2_tiles(exposure)
    threads = os.cpu_count() or 1
    n = max(threads, 4)
    for _ in range(max(args.warmup, 0) and 1):
        oracle_sample(params, tiles, min(n, 4), threads)
    secs, px = 0.0, 0
    for _ in range(args.steps):
        s, p = oracle_sample(params, tiles, n, threads)
        secs += s
        px += p
    total_px = sum(p.width_px * p.height_px for p in params)
    value = OUT_W * OUT_H * (px / args.steps / total_px) / (secs / args.steps) / 1e6
    sample = (f"each step renders {n} of the 49 C2 tiles with the C++ restatement of the reference CPU path "
              f"(faithful hit rule; the Rust reference cannot be built here), tiles in parallel on {threads} "
              f"threads; output Mpx/s scaled by tile pixels")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": C2_WORKLOAD + ", reference CPU path (no GPU used)", "tiles_per_step": n},
        "cpu_baseline": {"value": value, "unit": "Mpx/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 10; 1 for c4)")
    ap.add_argument("--warmup", type=int, default=None, help="untimed steps (default 3; 1 for c4)")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--tiles", type=int, default=0, help="render only the first N tiles of C2 (profiling)")
    ap.add_argument("--workload", choices=["c2", "c3", "c4", "fast"], default="c2",
                    help="c2: the headline configuration; c3: the mixed batch; c4: a 4096^2 RGB photograph at "
                         "supersample 4 through the film renderer; fast: the C2 tiles through the fast "
                         "approximation (c3, c4 and fast are reported, not the headline)")
    ap.add_argument("--film-side", type=int, default=4096, help="c4: side of the RGB photograph (4096 for C4)")
    ap.add_argument("--batch-gb", type=float, default=0.0,
                    help="c4: device GiB one batch of tiles may use (0: 70 %% of the free memory)")
    ap.add_argument("--profile-region", action="store_true",
                    help="bracket the timed replays with cudaProfilerStart/Stop")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 1 if args.workload == "c4" else 10
    if args.warmup is None:
        args.warmup = 1 if args.workload == "c4" else 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.workload == "fast":
        run_fast(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
