/* CPU oracle for the fgrain photon-transport and transmittance-scan path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates the reference's Rust CPU path in C++ so
 * that tests can check the CUDA library against it, and so that bench.py can time it as the
 * CPU baseline.  Nothing in the product links or calls it.
 *
 * Parity status: the geometric and development stages are pinned to the reference's own
 * inline known-answer tests (crystal.rs:238-282, bvh.rs:412-462, development.rs:197-265,
 * poisson.rs:141-165, optics.rs:206-245, transport.rs:195-237, transmittance.rs:181-221).
 * The random streams are NOT pinned: the reference draws from rand 0.8.8 StdRng (ChaCha12),
 * which cannot be built here; the oracle draws from Philox-4x32-10 instead (philox.h).
 */
#ifndef FG_ORACLE_H
#define FG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* GelatinOptics, optics.rs:41-60 */
typedef struct or_optics {
  double refractive_index;
  double absorption_coeff;
  double scattering_coeff;
  double anisotropy_g;
  double antihalation_reflectance;
  double antihalation_density;
} or_optics;

/* EmulsionConfig, emulsion.rs:14-37 (morphology: 0 cubic, 1 tabular, 2 octahedral) */
typedef struct or_emulsion_cfg {
  double width, height, depth;
  double r_min;
  double mean_crystal_radius;
  double size_variance;
  int32_t morphology;
  int32_t _pad;
  double tabular_aspect_ratio;
  or_optics optics;
  double base_sensitivity;
} or_emulsion_cfg;

/* ExposureConfig, transport.rs:15-28 */
typedef struct or_exposure_cfg {
  double photons_per_sq_um;
  double illumination_angle_rad;
  double crystal_absorption_coeff;
  uint32_t max_bounces;
  uint32_t _pad;
} or_exposure_cfg;

/* DevelopmentConfig, development.rs:12-27 */
typedef struct or_dev_cfg {
  uint32_t threshold_photons;
  uint32_t _pad;
  double filament_expansion;
  double clumping_proximity_factor;
  double developer_contrast;
} or_dev_cfg;

/* DevelopmentReport, development.rs:42-56 */
typedef struct or_dev_report {
  uint64_t total_crystals;
  uint64_t developed_crystals;
  uint64_t fixed_crystals;
  uint64_t total_clumps;
  uint64_t max_clump_size;
  double avg_clump_size;
} or_dev_report;

/* ScanConfig, transmittance.rs:32-48 (mode: 0 negative T, 1 positive 1-T, 2 optical density) */
typedef struct or_scan_cfg {
  uint32_t width_px;
  uint32_t height_px;
  uint32_t samples_per_pixel;
  int32_t mode;
  double silver_opacity;
} or_scan_cfg;

/* A crystal set in structure-of-arrays form (HalideCrystal, crystal.rs:21-50).  pos and dims
 * hold 3 doubles per crystal, quat holds (i, j, k, w).  The mutable fields (latent counts,
 * developed flag, clump id, filament expansion) live in the same struct so that the stages
 * can be chained exactly like the reference chains them. */
typedef struct or_crystals {
  size_t n;
  double* pos;
  double* dims;
  double* quat;
  double* sens;
  int32_t* morph;
  uint32_t* latent;
  uint8_t* developed;
  int64_t* clump;
  double* expansion;
} or_crystals;

/* Hit-selection rule.  FAITHFUL walks the reference's spatial-median BVH (bvh.rs:157-347) and
 * reports hits in its traversal order; a crystal counts when its geometry is hit and the
 * enclosing LEAF box is hit.  CANONICAL counts a crystal when its geometry is hit and its OWN
 * max_dim box (crystal.rs:106-133) is hit, and orders hits by (t_enter, crystal index); it does
 * not depend on how a BVH groups crystals, so a device LBVH can reproduce it exactly. */
enum { OR_FAITHFUL = 0, OR_CANONICAL = 1 };

/* One recorded photon segment: the state a bounce starts from. */
typedef struct or_segment {
  double origin[3];
  double dir[3];
  double step;
  double energy;
  uint32_t photon;
  uint32_t bounce;
} or_segment;

/* ---- known-answer entry points ---- */
int or_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
              uint32_t out[4]);
/* HalideCrystal::intersect_ray (crystal.rs:140-217); returns 1 on hit. */
int or_intersect_crystal(const double pos[3], const double dims[3], const double quat[4],
                         int32_t morph, double expansion, const double origin[3],
                         const double dir[3], double* t_enter, double* t_exit);
/* Builds the reference BVH over the set and returns the hits of one ray (faithful or
 * canonical).  Returns the number of hits (<= cap). */
int64_t or_ray_hits(const or_crystals* c, const double origin[3], const double dir[3], int mode,
                    uint32_t* idx_out, double* t0_out, double* t1_out, int64_t cap);
/* BVH::query_radius (bvh.rs:350-402); returns the number of results (<= cap). */
int64_t or_query_radius(const or_crystals* c, const double center[3], double radius,
                        uint32_t* out, int64_t cap);
/* Statistics of the reference BVH over the set: node count, depth, and stack drops. */
int or_bvh_stats(const or_crystals* c, int64_t* nodes, int64_t* depth);
/* FP64 transmittance of pixel windows (x0, y0, w, h) of a scan with the reference's rule, each
 * window under +-hstep on the opacity of crystal pidx[k]: three planes (base, plus, minus) per
 * window.  The tree over the developed crystals is built once.  Returns the doubles written. */
int64_t or_scan_windows(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg, uint64_t seed,
                        int threads, const double* sigma_c, int64_t nwin, const uint32_t* win, const uint32_t* pidx,
                        double hstep, double* T_out);
/* The reference tree (bvh.rs:157-295) over all crystals, or over the developed ones with their
 * expansion (the scan's tree): final index order (crystal indices) and the leaves in node order
 * (range in that order, box lo xyz hi xyz).  Returns the element count. */
int64_t or_bvh_export(const or_crystals* c, int developed_only, uint32_t* order, int64_t cap,
                      uint32_t* leaf_start, uint32_t* leaf_count, double* leaf_box, int64_t leaf_cap,
                      int64_t* nleaves);

/* GelatinOptics::sample_free_path (optics.rs:100-107) for one uniform xi. */
double or_free_path(const or_optics* o, double xi);
/* GelatinOptics::handle_antihalation_reflection (optics.rs:160-196) with its uniforms u[0..3]
 * (roulette, diffuse choice, u1, u2).  Returns 1 while the packet is alive. */
int or_antihalation(const or_optics* o, double* energy, double dir[3], const double u[4]);
/* Hits of many rays against the set (one BVH build): CSR offsets[n+1], ids, per-ray chord sums.
 * developed_only: test only developed crystals, with their expansion.  Returns total hits. */
int64_t or_rays_hits(const or_crystals* c, const double* origins, const double* dirs, int64_t n,
                     int mode, int developed_only, uint32_t* offsets, uint32_t* ids,
                     int64_t id_cap, double* chord_sum);

/* ---- stages ---- */
/* sample_poisson_3d (poisson.rs:14-132): returns the point count; writes at most cap points. */
int64_t or_sample_poisson(const double bounds[3], double r_min, uint32_t k, uint64_t seed,
                          double* pts, int64_t cap);
/* VirtualEmulsionLayer::synthesize (emulsion.rs:155-220).  Pass out->n = capacity. */
int64_t or_synthesize(const or_emulsion_cfg* cfg, uint64_t seed, or_crystals* out);

/* expose_emulsion (transport.rs:48-188) with the tile worker's nearest-pixel exposure closure
 * (image_pipeline.rs:949-958).  Counts are ADDED to c->latent.  When seg_out is not NULL the
 * segments are recorded (sorted by photon, bounce); *seg_n receives the total count even if it
 * exceeds seg_cap.  Returns the number of photons launched. */
int64_t or_expose(or_crystals* c, const or_emulsion_cfg* cfg, const float* tile, uint32_t tw,
                  uint32_t th, const or_exposure_cfg* ecfg, uint64_t seed, int mode,
                  int threads, or_segment* seg_out, int64_t seg_cap, int64_t* seg_n,
                  uint64_t* hits_out);

/* Replays recorded segments with the per-hit arithmetic of expose under hit rule `mode`
 * (OR_FAITHFUL: the reference's BVH walk and traversal order; OR_CANONICAL: own-box rule, sorted
 * by (t_enter, index)); counts are added to c->latent; hit lists (in absorption order) are written
 * CSR-style when offsets != NULL. */
int64_t or_replay_segments(or_crystals* c, const or_exposure_cfg* ecfg, uint64_t seed,
                           const or_segment* segs, int64_t nseg, int mode, uint32_t* offsets,
                           uint32_t* ids, int64_t id_cap);

/* develop_emulsion (development.rs:59-188): fills developed / clump / expansion. */
int or_develop(or_crystals* c, const or_dev_cfg* cfg, or_dev_report* rep);

/* scan_emulsion (transmittance.rs:65-171).  out receives the mode-mapped f32 buffer; image8
 * (optional) the 8-bit image.  sigma_c (optional) gives a per-crystal opacity in place of
 * cfg->silver_opacity.  T64 (optional) receives the FP64 pixel means.  ray_hits (optional)
 * receives, per ray (pixel-major, stratum-minor), the number of canonical/faithful hits. */
int or_scan(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
            uint64_t seed, int mode, int threads, const double* sigma_c, float* out,
            uint8_t* image8, double* T64, uint16_t* ray_hits);

/* The differentiable scan (the adjoint asked of this build; the reference scans with one opacity
 * and filters with fixed taps).  S = OTF_s(e T): T is or_scan's FP64 stratified mean
 * transmittance with per-crystal opacities sigma_c (NULL: scfg->silver_opacity for all), e an
 * exposure multiplier and OTF_s the scanner's separable 3-tap clamp-to-edge filter
 * (image_pipeline.rs:825-855) with taps (g, 1, g) / (1 + 2 g), g = exp(-1 / (2 s^2)); the
 * reference's taps (0.035, 0.93, 0.035) are s = 0.3904441347190481.  FP64 throughout. */
void or_otf_taps(double s, double taps[3], double dtaps[3]);
int or_scan_signal(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
                   uint64_t seed, int mode, int threads, const double* sigma_c, double exposure,
                   double otf_sigma, double* S, double* T);
/* Adjoint of or_scan_signal for an upstream gradient dL_dS (w*h): gradients with respect to the
 * per-crystal opacities (crystal-index order; undeveloped crystals get 0), the exposure
 * multiplier and the OTF width.  The forward is recomputed from the developed mask. */
int or_scan_backward(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
                     uint64_t seed, int mode, int threads, const double* sigma_c, double exposure,
                     double otf_sigma, const double* dL_dS, double* g_sigma, double* g_exposure,
                     double* g_otf);

/* Scan ray origins exactly as or_scan forms them (pixel-major, stratum-minor). */
int or_scan_ray_origins(const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg, uint64_t seed,
                        double* origins);

/* render_tile_cpu_full (image_pipeline.rs:924-987) + render_tile_cpu_density (:990-1014).
 * preset: 0 tri-x, 1 tri-x-1600, 2 t-max, 3 hp5.  tile is tw*th row-major exposure. */
typedef struct or_tile_report {
  uint64_t crystals;
  uint64_t developed;
  uint64_t clumps;
  uint64_t photons;
  uint64_t hits;
} or_tile_report;
int or_render_tile(int preset, double pixel_size_um, const float* tile, uint32_t tw, uint32_t th,
                   double exposure, double push, uint64_t tile_seed, int mode, int threads,
                   float* d_neg, or_tile_report* rep);

/* Scanner OTF, image_pipeline.rs:825-855 (3-tap, clamp to edge), on a float field. */
int or_scanner_otf(const float* in, uint32_t w, uint32_t h, const float taps[3], float* out);
/* Triangle-filter resize of a float field (the supersample downsample, image_pipeline.rs:
 * 315-330; separable tent filter whose support scales with the ratio). */
int or_resize_triangle(const float* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                       float* out);
/* Hann overlap blend of tiles into an image (image_pipeline.rs:593-649): returns d_norm. */
int or_blend_tiles(uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                   uint32_t ntiles, const uint32_t* desc /* ntiles x (tx,ty,x0,y0,tw,th) */,
                   const float* const* tiles, float* d_norm);

/* ---- image stages either side of the tile path (fg_oracle_film.cpp) ---- */
/* Panchromatic weights of a stock (image_pipeline.rs:265-284) and the luma of an RGB8 image
 * (image_pipeline.rs:286-294: round(clamp(r wr + g wg + b wb, 0, 255))). */
int or_luma_weights(const char* preset, float out[3]);
int or_luma(const uint8_t* rgb, uint32_t w, uint32_t h, const float wts[3], uint8_t* out);
/* The image crate's resize of a u8 image (filter 0 Triangle, 1 Lanczos3): vertical pass to f32,
 * horizontal pass, clamp and round to u8; a copy when the size is unchanged. */
int or_resize_u8(const uint8_t* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh, int filter,
                 uint8_t* out);
/* Camera gate and gelatin PSF (image_pipeline.rs:133-252): h_effective, zero outside the gate;
 * gate receives (top, bottom, left, right). */
int or_gelatin_psf(const uint8_t* src, uint32_t w, uint32_t h, float* heff, uint32_t gate[4]);
/* Grain amplitude of a stock (image_pipeline.rs:718-723). */
float or_film_base_nominal(const char* preset);
typedef struct or_finish_cfg {
  double grain_size_px; /* after scaling (image_pipeline.rs:365) */
  double strength;      /* effective strength (image_pipeline.rs:366) */
  double push;          /* effective push (image_pipeline.rs:369-375) */
  float base_nominal;
  int32_t scanner_otf;
} or_finish_cfg;
/* Everything after the tiles (image_pipeline.rs:593-891): Hann blend with weights, DoG low-pass
 * split, grain statistics, composite, scanner OTF and output gates, to a u8 image.  fields (may
 * be NULL) receives 5 planes: d_norm, d_low, grain, tone, scanned grain; stats (may be NULL)
 * receives high_mean, high_std, norm_factor. */
int or_film_finish(const or_finish_cfg* cfg, uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                   uint32_t ntiles, const uint32_t* desc, const float* const* tiles, const uint8_t* src,
                   const float* heff, uint8_t* out, float* fields, float* stats);

/* ---- the reference's wgpu tile model (fg_oracle_fast.cpp) ---- */
/* GpuTileParams (gpu.rs:18-37). */
typedef struct or_fast_params {
  double film_w, film_h, film_d;
  uint32_t width_px, height_px, samples_per_pixel, _pad0;
  double silver_opacity;
  uint64_t seed;
  double r_min, mean_crystal_radius, size_variance;
  uint32_t morphology, threshold_photons;
  double tabular_aspect_ratio, base_sensitivity, exposure, filament_expansion, clumping_proximity_factor;
} or_fast_params;
typedef struct or_fast_grid_t {
  uint32_t w, h, d;
  float cell_size;
} or_fast_grid_t;
/* The cell grid of a tile (gpu.rs:505-525). */
int or_fast_grid(const or_fast_params* p, or_fast_grid_t* g);
/* render_tile_all_gpu's shaders on the CPU: d_neg (width_px x height_px) and, when cells_out is not
 * NULL, the final grid cells (64 bytes each: pos, dims and expansion, quaternion, flags). */
int or_fast_tile(const or_fast_params* p, const float* tile, float* d_neg, void* cells_out);

#ifdef __cplusplus
}
#endif
#endif
