/* fgrain_cuda.h - C ABI of the GB300-native fgrain photon-transport and scan path.
 *
 * The library replaces, behind the reference's --gpu switch, the per-tile chain of the Rust
 * crate fgrain (paths are relative to that project):
 *   VirtualEmulsionLayer::synthesize   src/emulsion.rs:155
 *   expose_emulsion                    src/transport.rs:48   (re-exported src/lib.rs:34)
 *   develop_emulsion                   src/development.rs:59 (re-exported src/lib.rs:24)
 *   scan_emulsion                      src/transmittance.rs:65 (re-exported src/lib.rs:33)
 *   GpuEngine::render_tile_all_gpu     src/gpu.rs:491 (engine singleton src/gpu.rs:9-14)
 * with CPU-path physics (the reference's wgpu shaders run a different model).
 *
 * Conventions: plain C types, host pointers unless a name says "device", every entry point
 * returns fg_status.  An engine is safe to call from several threads: calls are serialised on
 * the engine's stream, like the reference's dispatch_lock (src/gpu.rs:169,503).  There is no
 * CPU fallback: on an error the caller decides (the reference falls back to its CPU chain,
 * src/image_pipeline.rs:535-558).  fg_last_error() returns the message of the last failure.
 */
#ifndef FGRAIN_CUDA_H
#define FGRAIN_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  1-6 mirror GpuError (src/error.rs:9-33) one to one. */
typedef enum fg_status {
  FG_OK = 0,
  FG_ERR_ADAPTER_NOT_FOUND = 1,     /* GpuError::AdapterNotFound: no CUDA device / bad index */
  FG_ERR_DEVICE_REQUEST_FAILED = 2, /* GpuError::DeviceRequestFailed: context / stream setup */
  FG_ERR_CHANNEL = 3,               /* GpuError::ChannelError: asynchronous completion failed */
  FG_ERR_BUFFER_MAP = 4,            /* GpuError::BufferMapError: host<->device copy failed */
  FG_ERR_BUFFER_RANGE = 5,          /* GpuError::BufferRangeError: size / capacity mismatch */
  FG_ERR_PIPELINE = 6,              /* GpuError::PipelineError: kernel launch or fault */
  FG_ERR_INVALID_ARG = 16,          /* bad pointer, size or configuration value */
  FG_ERR_OOM = 17,                  /* device allocation failed */
  FG_ERR_DEVICE_TIMEOUT = 18,       /* a bounded device wait gave up (error word set) */
  FG_ERR_DEVICE_OVERFLOW = 19       /* a fixed device capacity was exceeded (error word set) */
} fg_status;

typedef struct fg_engine fg_engine;
typedef struct fg_emulsion fg_emulsion;

typedef enum fg_morphology { FG_CUBIC = 0, FG_TABULAR = 1, FG_OCTAHEDRAL = 2 } fg_morphology;

/* GelatinOptics, src/optics.rs:41-60 */
typedef struct fg_optics {
  double refractive_index;
  double absorption_coeff;
  double scattering_coeff;
  double anisotropy_g;
  double antihalation_reflectance;
  double antihalation_density;
} fg_optics;

/* EmulsionConfig, src/emulsion.rs:14-37 (dimensions = width, height, depth in micrometres) */
typedef struct fg_emulsion_cfg {
  double width, height, depth;
  double r_min;
  double mean_crystal_radius;
  double size_variance;
  int32_t morphology; /* fg_morphology */
  int32_t _pad;
  double tabular_aspect_ratio;
  fg_optics optics;
  double base_sensitivity;
} fg_emulsion_cfg;

/* ExposureConfig, src/transport.rs:15-28 */
typedef struct fg_exposure_cfg {
  double photons_per_sq_um;
  double illumination_angle_rad;
  double crystal_absorption_coeff;
  uint32_t max_bounces;
  uint32_t _pad;
} fg_exposure_cfg;

/* DevelopmentConfig, src/development.rs:12-27 */
typedef struct fg_dev_cfg {
  uint32_t threshold_photons;
  uint32_t _pad;
  double filament_expansion;
  double clumping_proximity_factor;
  double developer_contrast;
} fg_dev_cfg;

/* DevelopmentReport, src/development.rs:42-56 */
typedef struct fg_dev_report {
  uint64_t total_crystals;
  uint64_t developed_crystals;
  uint64_t fixed_crystals;
  uint64_t total_clumps;
  uint64_t max_clump_size;
  double avg_clump_size;
} fg_dev_report;

/* ScanMode / ScanConfig, src/transmittance.rs:17-48 */
typedef enum fg_scan_mode { FG_SCAN_NEGATIVE = 0, FG_SCAN_POSITIVE = 1, FG_SCAN_OPTICAL_DENSITY = 2 } fg_scan_mode;
typedef struct fg_scan_cfg {
  uint32_t width_px;
  uint32_t height_px;
  uint32_t samples_per_pixel;
  int32_t mode; /* fg_scan_mode */
  double silver_opacity;
} fg_scan_cfg;

/* A crystal set on the host, structure of arrays in crystal-index order (HalideCrystal,
 * src/crystal.rs:21-50).  pos/dims: 3 doubles per crystal; quat: (i, j, k, w); morphology may be
 * NULL (then cfg->morphology applies to all). */
typedef struct fg_crystals_host {
  const double* pos;
  const double* dims;
  const double* quat;
  const double* sensitivity;
  const int32_t* morphology;
} fg_crystals_host;

/* Same layout for downloads (any pointer may be NULL). */
typedef struct fg_crystals_out {
  double* pos;
  double* dims;
  double* quat;
  double* sensitivity;
  int32_t* morphology;
} fg_crystals_out;

/* One photon segment as the reference's bounce loop sees it (src/transport.rs:101-185): the
 * position and direction a bounce starts from, its step length and the packet energy. */
typedef struct fg_segment {
  double origin[3];
  double dir[3];
  double step;
  double energy;
  uint32_t photon;
  uint32_t bounce;
} fg_segment;

/* Device time of the stages of the last call on an engine (CUDA events, milliseconds) and the
 * work it did.  Fields a call does not touch are zero. */
typedef struct fg_timings {
  double synth_ms, bvh_ms, transport_ms, develop_ms, scan_ms, post_ms, total_ms;
  uint64_t crystals, photons, hits, rays, developed, fallbacks;
  uint32_t kernel_launches;
  uint32_t error_word;
} fg_timings;

/* Process-wide cap on the device bytes this library holds at once through its own allocations
 * (0: none, the default).  An allocation past the cap fails with FG_ERR_OOM as a failed cudaMalloc
 * would, which lets callers and tests exercise the out-of-memory path without exhausting the GPU.
 * No counterpart in the reference. */
fg_status fg_set_device_budget(uint64_t bytes);

/* ---- engine (GpuEngine::new / get_gpu_engine, src/gpu.rs:9-14,174) ---- */
fg_status fg_engine_create(int device, fg_engine** out);
fg_status fg_engine_destroy(fg_engine* e);
const char* fg_last_error(const fg_engine* e);           /* message of the last failure */
const char* fg_engine_device_name(const fg_engine* e);   /* GpuEngine::adapter_name, gpu.rs:484 */
fg_status fg_engine_timings(const fg_engine* e, fg_timings* out);
const char* fg_status_string(fg_status s);

/* ---- presets (EmulsionConfig::tri_x_400 / tri_x_1600 / t_max_100 / hp5_plus,
 *      src/emulsion.rs:46-136); name: "tri-x", "tri-x-1600", "t-max", "hp5" ---- */
fg_status fg_emulsion_preset(const char* name, double width, double height, fg_emulsion_cfg* out);

/* ---- emulsions ---- */
/* VirtualEmulsionLayer::synthesize (src/emulsion.rs:155-220) on the device: Poisson-disk
 * positions (src/poisson.rs:14-132, column-parallel Bridson thinned to the reference sampler's
 * density) and crystal attributes, then the LBVH.  Crystal ids follow the Morton order of the
 * synthesis grid. */
fg_status fg_emulsion_synthesize(fg_engine* e, const fg_emulsion_cfg* cfg, uint64_t seed, fg_emulsion** out);
/* Upload a crystal set (for parity runs on exactly the oracle's crystals).  The device keeps the
 * FP64 values for exact predicates and builds the Morton-ordered LBVH. */
fg_status fg_emulsion_upload(fg_engine* e, const fg_emulsion_cfg* cfg, const fg_crystals_host* c,
                             size_t n, fg_emulsion** out);
fg_status fg_emulsion_destroy(fg_engine* e, fg_emulsion* em);
fg_status fg_emulsion_count(const fg_emulsion* em, size_t* n);
fg_status fg_emulsion_download(fg_engine* e, const fg_emulsion* em, fg_crystals_out* out);
/* Latent counts (HalideCrystal::latent_photons, src/crystal.rs:41), crystal-index order. */
fg_status fg_emulsion_get_counts(fg_engine* e, const fg_emulsion* em, uint32_t* counts);
fg_status fg_emulsion_set_counts(fg_engine* e, fg_emulsion* em, const uint32_t* counts);
/* Developed flag, clump id (-1 when none) and filament expansion per crystal (any may be NULL). */
fg_status fg_emulsion_get_development(fg_engine* e, const fg_emulsion* em, uint8_t* developed,
                                      int64_t* clump, double* expansion);
/* Fix the developed mask and expansions (a scan with a fixed developed mask). */
fg_status fg_emulsion_set_development(fg_engine* e, fg_emulsion* em, const uint8_t* developed,
                                      const double* expansion);

/* ---- stages ---- */
/* expose_emulsion (src/transport.rs:48-188) with the tile worker's exposure closure: tile is
 * tw*th row-major float, sampled at the nearest pixel (src/image_pipeline.rs:949-958).  Counts
 * are added to the emulsion's latent counts, like record_absorption (src/crystal.rs:221). */
fg_status fg_expose_emulsion(fg_engine* e, fg_emulsion* em, const float* tile, uint32_t tw,
                             uint32_t th, const fg_exposure_cfg* cfg, uint64_t seed);

/* develop_emulsion (src/development.rs:59-188).  report may be NULL. */
fg_status fg_develop_emulsion(fg_engine* e, fg_emulsion* em, const fg_dev_cfg* cfg,
                              fg_dev_report* report);

/* scan_emulsion (src/transmittance.rs:65-171).  out: width*height mode-mapped floats;
 * image8 (may be NULL): the 8-bit image.  sigma_per_crystal (may be NULL): per-crystal silver
 * opacity in crystal-index order, replacing cfg->silver_opacity. */
fg_status fg_scan_emulsion(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg,
                           uint64_t seed, const float* sigma_per_crystal, float* out,
                           uint8_t* image8);

/* ---- replay (parity) ---- */
/* Differentiable scan (scan_emulsion, src/transmittance.rs:65-171, followed by the scanner OTF of
 * src/image_pipeline.rs:825-855).  signal = OTF_s(exposure * T) per pixel, where T is the scanned
 * transmittance (Negative mode; cfg->mode is ignored) with per-crystal opacities sigma_per_crystal
 * (crystal-index order; NULL: cfg->silver_opacity for all) and OTF_s the separable 3-tap
 * clamp-to-edge filter with taps (g, 1, g) / (1 + 2 g), g = exp(-1 / (2 s^2));
 * s = 0.3904441347190481 reproduces the reference's taps (0.035, 0.93, 0.035).  signal and
 * transmittance (width*height floats each) may be NULL, not both. */
fg_status fg_scan_signal(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg, uint64_t seed,
                         const float* sigma_per_crystal, double exposure, double otf_sigma, float* signal,
                         float* transmittance);
/* Hand-written adjoint of fg_scan_signal (no counterpart in the reference): for the upstream
 * gradient dL_dsignal (width*height) returns dL/dsigma per crystal (crystal-index order; 0 for
 * undeveloped crystals), dL/dexposure and dL/dotf_sigma.  Any output may be NULL.  The forward is
 * recomputed from the developed mask; no intermediate of an earlier call is kept. */
fg_status fg_scan_backward(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg, uint64_t seed,
                           const float* sigma_per_crystal, double exposure, double otf_sigma,
                           const float* dL_dsignal, float* dL_dsigma, double* dL_dexposure,
                           double* dL_dotf_sigma);

/* ---- image stages around the tile path (host arrays, row-major floats) ---- */
/* Hann overlap blend of tile densities into d_norm (src/image_pipeline.rs:593-649): desc holds
 * (tx, ty, x_start, y_start, tw, th) per tile in grid order (index ty * ntx + tx, the order of
 * src/image_pipeline.rs:377-424); tiles[t] is tile t's tw*th density. */
fg_status fg_blend_tiles(fg_engine* e, uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                         uint32_t ntiles, const uint32_t* desc, const float* const* tiles, float* d_norm);
/* Scanner OTF (src/image_pipeline.rs:825-855): separable 3-tap clamp-to-edge filter; taps NULL
 * means the reference's (0.035, 0.93, 0.035). */
fg_status fg_scanner_otf(fg_engine* e, const float* in, uint32_t w, uint32_t h, const float* taps, float* out);
/* Supersample downsample (src/image_pipeline.rs:315-330): Triangle filter of the image crate,
 * vertical pass then horizontal, w x h -> ow x oh. */
fg_status fg_resize_triangle(fg_engine* e, const float* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                             float* out);

/* ---- whole photographs: the film renderer around the tile path ---- */
/* FilmRenderOptions (src/image_pipeline.rs:18-101).  out_w = out_h = 0 keeps the input size; one
 * of them 0 keeps the aspect ratio (output_resolution, src/image_pipeline.rs:306-313).  eberhard
 * has no effect (the reference's halo term is zero, src/image_pipeline.rs:789). */
typedef struct fg_film_options {
  const char* preset;      /* "tri-x", "t-max", "hp5", "tri-x-1600", "caffenol", ... */
  double grain_size_px;    /* 2.2 */
  double grain_strength;   /* 1.0 */
  double exposure;         /* 1.0 */
  int32_t color;           /* 0: black and white; 1: three dye layers (needs 3 channels) */
  uint32_t out_w, out_h;   /* 0, 0 */
  uint32_t tile_size;      /* 320 */
  uint64_t seed;           /* 42 */
  int32_t auto_scale;      /* 0 */
  uint32_t reference_res;  /* 6000 */
  double scale;            /* 1.0 */
  uint32_t supersample;    /* 1 (1 to 4) */
  int32_t scanner_otf;     /* 1 */
  double push;             /* 0 */
  double eberhard;         /* 1.0 */
  uint64_t batch_bytes;    /* device bytes one batch of tiles may use; 0: 70 % of the free memory.
                              Larger images run as several batches, with identical results. */
} fg_film_options;

typedef struct fg_film_report {  /* ImageProcessReport (src/image_pipeline.rs:97-105) */
  uint32_t in_w, in_h, out_w, out_h;
  uint64_t total_tiles, total_crystals, photons;
  double elapsed_seconds;
  uint64_t developed_crystals, total_clumps;
  /* device time (CUDA events) of the image stages before the tiles (resize, gate, PSF), of the
   * tile batches (gather, run, density copy) and of the finish (blend to u8, downscale) */
  double prep_ms, tiles_ms, finish_ms;
} fg_film_report;

/* The reference's defaults (FilmRenderOptions::default, src/image_pipeline.rs:82-101). */
void fg_film_options_default(fg_film_options* o);
fg_status fg_film_output_size(const fg_film_options* o, uint32_t in_w, uint32_t in_h, uint32_t* out_w,
                              uint32_t* out_h);
/* render_film_black_and_white_tiled / render_film_color_tiled (src/image_pipeline.rs:299-891,
 * 1017-1085) with every stage on the device: pixels is a u8 image of `channels` (1 gray, 3 RGB
 * interleaved) channels, out receives out_w x out_h x (color ? 3 : 1) bytes.  A gray render of an
 * RGB image takes the stock's panchromatic luma first.  The tiles of all layers run as one batch,
 * or as consecutive batches within options->batch_bytes. */
fg_status fg_render_film(fg_engine* e, const uint8_t* pixels, uint32_t w, uint32_t h, uint32_t channels,
                         const fg_film_options* options, uint8_t* out, fg_film_report* report);

/* Stages of the renderer, for parity checks and for callers that compose their own pipeline. */
/* convert_to_panchromatic_luma (src/image_pipeline.rs:259-296) of an RGB8 image. */
fg_status fg_panchromatic_luma(fg_engine* e, const uint8_t* rgb, uint32_t w, uint32_t h, const char* preset,
                               uint8_t* out);
/* image::imageops::resize of a u8 image (src/image_pipeline.rs:324-328, 333-342): the image
 * crate's separable filter, vertical pass to f32 then horizontal pass, clamped and rounded. */
#define FG_FILTER_TRIANGLE 0
#define FG_FILTER_LANCZOS3 1
fg_status fg_resize_u8(fg_engine* e, const uint8_t* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                       int32_t filter, uint8_t* out);
/* apply_camera_and_gelatin_optics (src/image_pipeline.rs:133-252): h_effective of a u8 image
 * (zero outside the camera gate); gate (may be NULL) receives top, bottom, left, right. */
fg_status fg_gelatin_psf(fg_engine* e, const uint8_t* src, uint32_t w, uint32_t h, float* h_eff, uint32_t* gate);
/* Everything after the tiles (src/image_pipeline.rs:593-891): Hann blend with the weight sums,
 * low-frequency split, grain statistics, sensitometric composite, scanner OTF and output gates.
 * desc and tiles as in fg_blend_tiles; src is the u8 image at the render size, h_eff its PSF.
 * fields (may be NULL) receives 5 planes of out_w x out_h floats: d_norm, d_low, grain, tone,
 * scanned grain; stats (may be NULL) receives 4 floats: high_mean, high_std, norm_factor, 0. */
typedef struct fg_finish_cfg {
  const char* preset;      /* picks the grain amplitude (src/image_pipeline.rs:718-723) */
  double grain_size_px;    /* after scaling (src/image_pipeline.rs:365) */
  double grain_strength;   /* effective strength (src/image_pipeline.rs:366) */
  double push;             /* effective push (src/image_pipeline.rs:369-375) */
  int32_t scanner_otf;
  int32_t _pad;
} fg_finish_cfg;
fg_status fg_film_finish(fg_engine* e, const fg_finish_cfg* cfg, uint32_t out_w, uint32_t out_h, uint32_t tile_step,
                         uint32_t pad, uint32_t ntiles, const uint32_t* desc, const float* const* tiles,
                         const uint8_t* src, const float* h_eff, uint8_t* out, float* fields, float* stats);

/* Replays recorded segments with the exact hit rule and FP64 per-hit arithmetic.  Latent counts
 * are added to the emulsion.  Hit lists are returned CSR style: offsets[nseg+1], ids (crystal
 * indices in canonical order); *nhits receives the total even when it exceeds id_cap. */
fg_status fg_replay_segments(fg_engine* e, fg_emulsion* em, const fg_exposure_cfg* cfg,
                             uint64_t seed, const fg_segment* segs, size_t nseg,
                             uint32_t* offsets, uint32_t* ids, size_t id_cap, size_t* nhits);
/* Hits of arbitrary rays against the developed crystals (exact rule), CSR style, plus the
 * per-ray sum of chord lengths (may be NULL). */
fg_status fg_replay_rays(fg_engine* e, const fg_emulsion* em, const double* origins,
                         const double* dirs, size_t nrays, int developed_only, uint32_t* offsets,
                         uint32_t* ids, size_t id_cap, size_t* nhits, double* chord_sum);
/* The device's copy of the reference tree (BVH::build, bvh.rs:157-295) over the emulsion's crystals
 * (developed_only = 0: the transport's tree) or over its developed crystals with their expansion
 * (developed_only = 1: the scan's tree, transmittance.rs:86-89).  order receives the crystal ids in
 * the tree's final index order (BVH::indices), leaves 2 words per leaf (first index, count) sorted
 * by first index, leaf_boxes 6 doubles per leaf (lo xyz, hi xyz); at most cap entries each (any
 * may be NULL).  *nelem and *nleaves receive the totals. */
fg_status fg_emulsion_reference_tree(fg_engine* e, const fg_emulsion* em, int developed_only, uint32_t* order,
                                     uint32_t* leaves, double* leaf_boxes, size_t cap, size_t* nelem,
                                     size_t* nleaves);
/* Per-ray hit counts of the production scan kernel (pixel-major, stratum-minor). */
fg_status fg_scan_ray_hits(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg* cfg,
                           uint64_t seed, uint16_t* ray_hits);

/* ---- tiles: the drop-in for GpuEngine::render_tile_all_gpu (src/gpu.rs:491-938) ---- */

/* Per-tile parameters: GpuTileParams (src/gpu.rs:18-37) with the same meaning, followed by the
 * CPU-path physics of the reference's tile worker (src/image_pipeline.rs:924-1014) that
 * GpuTileParams does not carry.  Seeds follow the tile worker: synthesis `seed`, exposure
 * `seed + 1`, scan `seed + 2`; photons per um^2 = photons_per_sq_um * max(exposure, 0.05). */
typedef struct fg_tile_params {
  double film_w, film_h, film_d;
  uint32_t width_px, height_px;
  uint32_t samples_per_pixel;
  uint32_t threshold_photons;
  double silver_opacity;
  uint64_t seed;
  double r_min, mean_crystal_radius, size_variance;
  int32_t morphology;
  int32_t _pad0;
  double tabular_aspect_ratio, base_sensitivity, exposure;
  double filament_expansion, clumping_proximity_factor;
  fg_optics optics;
  double photons_per_sq_um;
  double illumination_angle_rad;
  double crystal_absorption_coeff;
  uint32_t max_bounces;
  uint32_t _pad1;
} fg_tile_params;

/* Fills the parameters the reference's CPU tile worker would use for a tile of tw x th pixels of
 * pixel_size_um micrometres (stock selection image_pipeline.rs:925-938, exposure config :942-947,
 * development :963-976 with the effective push of :369-375, scan :996-1002). */
fg_status fg_tile_params_preset(const char* preset, double pixel_size_um, uint32_t tw, uint32_t th,
                                double exposure, double push, uint64_t tile_seed, fg_tile_params* out);

/* Plain per-tile path: one tile from exposure (tw*th floats) to negative density
 * d = -log10(clamp(T, 1e-4, 1)) + 0.05 (src/image_pipeline.rs:1007-1011); blocking; device
 * buffers are made and freed inside the call, like the reference engine's per-call buffers. */
fg_status fg_render_tile(fg_engine* e, const float* tile, const fg_tile_params* params, float* d_neg);

/* ---- batches: many tiles in one graph-captured sequence of launches ---- */
typedef struct fg_batch fg_batch;
typedef struct fg_batch_options {
  int32_t use_graph;              /* capture the run into a CUDA graph (default in NULL options) */
  int32_t autotune;               /* time launch shapes when the plan is made */
  uint32_t transport_threads;     /* 0: default */
  uint32_t transport_blocks;      /* 0: default */
  uint32_t scan_bin_px;           /* 0: default */
  uint32_t synth_wait_limit;      /* polls before a synthesis column stops waiting for its
                                     neighbours (about 64 ns each; 0: 2^22) */
  int32_t wait_probe;             /* failure drill: nonzero makes every synthesis column also wait
                                     on a device flag that nothing sets, so the bounded wait runs
                                     out and the run fails with FG_ERR_DEVICE_TIMEOUT */
  uint32_t _pad;
} fg_batch_options;

typedef struct fg_batch_stats {
  double synth_ms, bvh_ms, transport_ms, develop_ms, scan_ms, total_ms;
  uint64_t crystals, photons, rays, pixels;
  uint64_t hits;            /* absorbing photon-crystal hits in transport */
  uint64_t scan_hits;       /* scanner ray-crystal hits */
  uint64_t scan_fallbacks;  /* scanner decisions taken in FP64 */
  uint32_t transport_threads, transport_blocks, scan_bin_px, graph, kernel_launches, _pad;
  uint64_t developed;       /* developed crystals (development.rs:79-84) */
  uint64_t clumps;          /* clumps: connected components of developed crystals (development.rs:107-108) */
  uint64_t cells;           /* synthesis grid cells of all tiles (r_min / sqrt(3) edge, poisson.rs:25-31) */
  double bridson_ms;        /* the Bridson kernel alone (the done-flag clear and its launch; CUDA events) */
} fg_batch_stats;

fg_status fg_batch_create(fg_engine* e, const fg_tile_params* tiles, uint32_t ntiles,
                          const fg_batch_options* options, fg_batch** out);
fg_status fg_batch_destroy(fg_batch* b);
/* Copies every tile's exposure (width_px * height_px floats each) from the host. */
fg_status fg_batch_set_exposure(fg_batch* b, const float* const* tiles);
/* Device addresses of a tile's exposure input and density output (valid for the batch's life). */
fg_status fg_batch_exposure_device(fg_batch* b, uint32_t tile, float** ptr);
fg_status fg_batch_density_device(fg_batch* b, uint32_t tile, const float** ptr);
/* Enqueues one run on the engine stream (returns at once); wait for it with fg_batch_wait. */
fg_status fg_batch_run(fg_batch* b);
fg_status fg_batch_wait(fg_batch* b, fg_batch_stats* stats);
fg_status fg_batch_get_density(fg_batch* b, float* const* outs);
/* The synthesized crystals of one tile after a run, with their latent counts, developed flags and
 * expansions (any pointer may be NULL); *n receives the tile's crystal count. */
fg_status fg_batch_tile_crystals(fg_batch* b, uint32_t tile, fg_crystals_out* out, uint32_t* counts,
                                 uint8_t* developed, double* expansion, size_t cap, size_t* n);
/* Replays the batch `steps` times back to back on the engine stream; *ms receives the device time
 * between CUDA events recorded before the first and after the last replay. */
fg_status fg_batch_time(fg_batch* b, uint32_t steps, double* ms);
/* Page-locked host memory for fast host<->device copies of exposure and density tiles. */
fg_status fg_host_alloc(size_t bytes, void** ptr);
fg_status fg_host_free(void* ptr);
/* Convenience: plan, copy in, run, copy out and free (no graph). */
fg_status fg_render_batch(fg_engine* e, const fg_tile_params* tiles, uint32_t ntiles,
                          const float* const* exposure, float* const* d_neg);

/* ---- fast approximation: the reference's wgpu tile model ---- */
/* The compute shaders of GpuEngine::render_tile_all_gpu (src/gpu.rs:491-938,
 * src/shaders/{poisson,develop,scan}.wgsl) as CUDA kernels: one jittered crystal per grid cell
 * relaxed against its neighbours, a per-crystal Poisson photon count from the local pixel instead
 * of photon transport, neighbour clumping, and a scan of the 5 x 5 cell columns around each ray.
 * A different, cheaper model than fg_render_tile's CPU-path physics.  Uses of fg_tile_params:
 * film size, pixels, samples per pixel, silver opacity, seed, r_min, radius distribution,
 * morphology, aspect ratio, sensitivity, exposure, filament expansion and clumping factor. */
/* GpuTileParams of the reference's GPU branch (src/image_pipeline.rs:455-518). */
fg_status fg_tile_params_fast_preset(const char* preset, double pixel_size_um, uint32_t tw, uint32_t th,
                                     double exposure, double push, uint64_t tile_seed, fg_tile_params* out);
/* The tile's cell grid (src/gpu.rs:505-525): dims[3] = (w, h, d), cells of *cell_size um. */
fg_status fg_fast_grid(const fg_tile_params* p, uint32_t* dims, float* cell_size);
/* d_neg of ntiles tiles in one set of launches; cells (may be NULL, or hold NULL entries) receives
 * each tile's final grid, 64 bytes per cell: position (4 floats), half-dimensions and expansion
 * (4 floats), quaternion (4 floats), flags (occupied, morphology, developed, photons). */
fg_status fg_render_tiles_fast(fg_engine* e, const fg_tile_params* params, uint32_t ntiles, const float* const* tiles,
                               float* const* d_neg, void* const* cells);
fg_status fg_render_tile_fast(fg_engine* e, const float* tile, const fg_tile_params* params, float* d_neg,
                              void* cells);

/* ---- Scan without device allocation ---------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot let this library allocate device
 * memory (a host that runs under a fixed device-memory budget or its own pool allocator, a plugin
 * inside such a host, code that must avoid the device-wide synchronisation of cudaMalloc /
 * cudaFree): the scan of fg_scan_emulsion over a crystal set and into an image that the caller
 * already holds in device memory.  It calls no cudaMalloc, cudaFree or allocating library
 * routine; its scratch is one file-scope device array of FG_STATIC_SCAN_SCRATCH_BYTES that every
 * GPU loading this library holds until the process exits, shared by all calls on that device. */
#define FG_STATIC_SCAN_MAX_CRYSTALS 1048576u /* crystals per call */
#define FG_STATIC_SCAN_MAX_DEVELOPED 32768u  /* developed crystals per call */
#define FG_STATIC_SCAN_MAX_BINS 16384u       /* scan bins (bin_px x bin_px pixels each) per call */
#define FG_STATIC_SCAN_MAX_ITEMS 1048576u    /* (developed crystal, bin) entries per call */
#define FG_STATIC_SCAN_SCRATCH_BYTES 17360128u

/* A crystal set in device memory, in crystal-index order (any order gives the same image). */
typedef struct fg_device_crystals {
  const float* a;           /* n x 4, 16-byte aligned: position x, y, z (um), sensitivity */
  const float* q;           /* n x 4, 16-byte aligned: unit quaternion i, j, k, w */
  const float* d;           /* n x 4, 16-byte aligned: dims x, y, z (um), morphology (int32 bits) */
  const double* pos64;      /* n x 3 FP64 positions, or NULL to decide ties from the floats */
  const double* dims64;     /* n x 3, given together with pos64 */
  const double* quat64;     /* n x 4, given together with pos64 */
  const uint8_t* developed; /* n development flags */
  const double* expansion;  /* n development expansions (development.rs:156-168) */
  uint64_t n;
} fg_device_crystals;

/* Scans `crystals` like fg_scan_emulsion over a film of film->width x film->height x film->depth
 * um (the other fields of film are ignored).  out (width*height floats) and image8 (width*height
 * bytes, may be NULL) are device pointers; work runs on `stream` (a cudaStream_t; NULL is the
 * legacy default stream) and the call returns when it has finished.  Requests with more than
 * FG_STATIC_SCAN_MAX_CRYSTALS crystals or FG_STATIC_SCAN_MAX_DEVELOPED developed ones, or needing
 * more than FG_STATIC_SCAN_MAX_BINS bins or FG_STATIC_SCAN_MAX_ITEMS entries, fail with
 * FG_ERR_INVALID_ARG before any output is written.  On failure a message is copied to `message` (message_len bytes,
 * may be NULL).  The first call on a device looks up the scratch's device address
 * (cudaGetSymbolAddress).  Every call on a device
 * shares the scratch, which keeps the last call's contents; each call clears what must start at
 * zero.  Calls whose GPU work overlapped would race on the scratch and give wrong images, so the
 * library serialises them: a call holds a per-device lock until its GPU work has finished (also
 * when it fails), and concurrent calls from other host threads wait.  a, q, d must be 16-byte
 * aligned, pos64, dims64, quat64 and expansion 8-byte aligned and out 4-byte aligned; anything
 * else fails with FG_ERR_INVALID_ARG before the GPU is touched. */
fg_status fg_scan_crystals_static(const fg_device_crystals* crystals, const fg_emulsion_cfg* film,
                                  const fg_scan_cfg* cfg, uint64_t seed, float* out, uint8_t* image8,
                                  void* stream, char* message, size_t message_len);

/* ---- Host helper of the command-line tool (no GPU involved) ---- */

/* Reverses the PNG row filters (ISO/IEC 15948:2003 section 9) in place, for the tool that reads
 * photographs the way image::open does (src/image_pipeline.rs:1141, the image crate's PNG codec):
 * rows holds h scanlines of 1 + stride bytes (the filter-type byte, then the filtered bytes); bpp
 * is the bytes per complete pixel (1 for bit depths below 8).  On return every filter byte is 0
 * and the scanlines hold the reconstructed bytes.  An unknown filter type gives
 * FG_ERR_INVALID_ARG (rows before it are already reconstructed). */
fg_status fg_png_unfilter(uint8_t* rows, uint32_t h, uint32_t stride, uint32_t bpp);

/* JPEG files as image::open and ImageBuffer::save handle them (src/image_pipeline.rs:1141, 1091,
 * 1114; the image crate's `jpeg` feature, Cargo.toml:13).  Reading: sequential Huffman-coded DCT
 * (SOF0, SOF1), 8-bit samples, one component (gray) or three (YCbCr; RGB when an Adobe marker
 * says so), any sampling factors and restart intervals; progressive, arithmetic-coded, lossless,
 * 12-bit and CMYK files give FG_ERR_INVALID_ARG with the reason in msg.  fg_jpeg_info reads the
 * header only: width, height and channels (1 or 3, what fg_jpeg_decode writes per pixel).
 * fg_jpeg_decode writes h rows of w * channels bytes (gray, or R, G, B) into out, cap bytes.
 * fg_jpeg_encode writes baseline JFIF at quality 1..100 (the example tables of ITU T.81 Annex K
 * scaled as the IJG library does; the image crate's default is 75): channels 1 (gray) or 3 (RGB,
 * stored as YCbCr).  options: the chroma subsampling (FG_JPEG_SUBSAMPLE_*, 4:2:0 when 0, what
 * writing an image file uses), FG_JPEG_SEPARATE_SCANS for one scan per component instead of one
 * interleaved scan, and FG_JPEG_RESTART(n) for a restart marker every n MCUs (n < 65536).  *len
 * receives the file's size; when it exceeds cap nothing useful is written and FG_ERR_INVALID_ARG
 * is returned (call again with *len bytes).  No GPU counterpart: host code of the command-line
 * tool. */
#define FG_JPEG_SUBSAMPLE_420 0x0u
#define FG_JPEG_SUBSAMPLE_422 0x1u
#define FG_JPEG_SUBSAMPLE_444 0x2u
#define FG_JPEG_SEPARATE_SCANS 0x4u
#define FG_JPEG_RESTART(n) ((uint32_t)(n) << 16)
fg_status fg_jpeg_info(const uint8_t* data, size_t n, uint32_t* w, uint32_t* h, uint32_t* channels, char* msg,
                       size_t msg_cap);
fg_status fg_jpeg_decode(const uint8_t* data, size_t n, uint8_t* out, size_t cap, char* msg, size_t msg_cap);
fg_status fg_jpeg_encode(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint32_t quality,
                         uint32_t options, uint8_t* out, size_t cap, size_t* len);

/* WebP files (the image crate's `webp` feature, Cargo.toml:13; its encoder writes lossless
 * WebP): the lossless format (VP8L) in a RIFF container.  Reading covers the whole lossless
 * format (predictor, colour and subtract-green transforms, colour indexing with pixel bundling,
 * colour cache, meta prefix codes, backward references); lossy (VP8) and animated files give
 * FG_ERR_INVALID_ARG with the reason in msg.  fg_webp_info: width, height and the header's alpha
 * hint.  fg_webp_decode writes h rows of w RGBA pixels (4 bytes each) into rgba, cap bytes.
 * fg_webp_encode takes channels 1 (gray, stored as R = G = B), 3 (RGB) or 4 (RGBA) and the tools
 * of the format to use (FG_WEBP_* bits; FG_WEBP_DEFAULT is what writing an image file uses; the
 * others exist to exercise every decoding path).  *len as for fg_jpeg_encode. */
#define FG_WEBP_SUBTRACT_GREEN 0x01u
#define FG_WEBP_PREDICTOR 0x02u
#define FG_WEBP_COLOR_TRANSFORM 0x04u
#define FG_WEBP_PALETTE 0x08u /* colour indexing when the image has at most 256 colours */
#define FG_WEBP_COLOR_CACHE 0x10u
#define FG_WEBP_BACKREFS 0x20u
#define FG_WEBP_META_CODES 0x40u
#define FG_WEBP_ALL_MODES 0x80u /* predictor modes assigned in turn rather than chosen */
#define FG_WEBP_DEFAULT (FG_WEBP_SUBTRACT_GREEN | FG_WEBP_PREDICTOR | FG_WEBP_COLOR_CACHE | FG_WEBP_BACKREFS)
fg_status fg_webp_info(const uint8_t* data, size_t n, uint32_t* w, uint32_t* h, uint32_t* has_alpha, char* msg,
                       size_t msg_cap);
fg_status fg_webp_decode(const uint8_t* data, size_t n, uint8_t* rgba, size_t cap, char* msg, size_t msg_cap);
fg_status fg_webp_encode(const uint8_t* px, uint32_t w, uint32_t h, uint32_t channels, uint32_t options,
                         uint8_t* out, size_t cap, size_t* len);

#ifdef __cplusplus
}
#endif
#endif /* FGRAIN_CUDA_H */
