// Device code of the transmittance scan (transmittance.rs:65-171).
//
// Scanner rays are vertical (origin (x, y, depth + 0.1), direction -z), so the scan is a 2D
// problem.  The reference walks a tree over the developed crystals (transmittance.rs:86-89,
// bvh.rs:300-347) and counts every crystal of every leaf whose box the ray hits by its geometry
// alone; a leaf box is hit by a vertical ray iff it contains the ray's (x, y) strictly
// (bvh.rs:96-124 with inv_dir = (inf, inf, -1)).  So a ray hits crystal s iff its geometry is hit
// and (x, y) lies strictly inside the box of s's leaf in that tree (built on the device, see
// fg_rtree.cuh).  The image is cut into bins of bin_px x bin_px pixels; every developed crystal is
// listed in the bins its leaf box overlaps; one CTA scans one bin: it stages the bin's crystals in
// shared memory, pre-transformed for vertical rays and relative to the bin corner, then each
// thread traces one stratum ray against them.
//
// Hit decisions are exact: each FP32 decision quantity carries a per-crystal error bound; when
// a margin falls inside it the ray/crystal pair is re-evaluated with the reference's FP64
// expressions (fg_device.cuh).  Chord lengths are summed in 64-bit fixed point (2^-40 um), so the
// sum is exact, deterministic and independent of list order.  The per-pixel mean over strata and
// the density conversion are FP64.
#pragma once
#include "fg_device.cuh"
#include "fg_rtree.cuh"

namespace fg {

constexpr int SCAN_CH = 128;        // crystals staged per pass
constexpr int SCAN_THREADS = 256;   // rays per CTA (bin_px^2 * strata)

// Bin-independent part of a developed crystal's staging, derived once per crystal in FP64 and
// rounded (k_scan_prep): each bin that lists the crystal only adds its centre relative to the
// bin's corner.  160 bytes, read with vector loads.
struct __align__(16) ScanPrep {
  // Centre x, y (um) as the scan sees it, and the x and y extent of the crystal's leaf box in the
  // scan's tree, as float pairs (hi + lo): x, y, leaf x0, x1, y0, y1.
  float ch[6], cl[6];
  float g[21];     // per-kind terms (see stage_crystal)
  float m, delta, err, sig;
  int kind;
  int pad_[2];
};
static_assert(sizeof(ScanPrep) == 160, "ScanPrep layout");

struct ScanTile {
  const ScanPrep* prep;  // staging of developed crystals (null: derived in each bin)
  unsigned long long slot_base;  // first crystal slot of this tile in a batch
  const float4* a;
  const float4* q;
  const float4* d;
  const double* pos64;
  const double* dims64;
  const double* quat64;
  const uint8_t* developed;
  const double* exp64;
  const double* lbox64;    // the scan tree's node boxes (lo xyz, hi xyz; tile-local node ids)
  const uint32_t* leafof;  // per crystal slot: its leaf in the scan tree
  const float* sigma_c;  // per crystal (Morton order) or null
  const uint32_t* bin_off;
  const uint32_t* bin_items;
  float* out;
  uint8_t* image8;
  float* d_neg;
  uint16_t* ray_hits;
  double pw, ph, z0;
  float jxh, jxl, jyh, jyl;  // pw / (g 2^24), ph / (g 2^24) as float pairs: one unit of the jitter
  uint64_t seed;
  unsigned long long bin_base;  // first global bin of this tile
  uint32_t w, h, g, spp, bin_px, nbx, nby, n;
  float sigma;
  int mode;
  uint32_t items_cap;  // entries of bin_items; lists past it were dropped (overflow flagged)
};

// Sets the jitter units of a tile whose pw, ph and g are set (host side, once per tile).
inline void set_jitter_units(ScanTile& t) {
  const double scale = 1.0 / (static_cast<double>(t.g) * 16777216.0);
  const double ux = t.pw * scale, uy = t.ph * scale;
  t.jxh = static_cast<float>(ux);
  t.jxl = static_cast<float>(ux - static_cast<double>(t.jxh));
  t.jyh = static_cast<float>(uy);
  t.jyl = static_cast<float>(uy - static_cast<double>(t.jyh));
}

// Stratum ray origin in FP64 exactly as the reference forms it (transmittance.rs:102-120).
__device__ __forceinline__ void scan_origin64(const ScanTile& t, uint32_t px, uint32_t py,
                                              uint32_t sx, uint32_t sy, double& ox, double& oy) {
  const uint64_t ps = t.seed + static_cast<uint64_t>(px) * 0x9E3779B97F4A7C15ull +
                      static_cast<uint64_t>(py) * 0xC6A4A7935BD1E995ull;
  const P4 r = philox(sy * t.g + sx, 0, 0, TAG_SCAN, static_cast<uint32_t>(ps), static_cast<uint32_t>(ps >> 32));
  const double gd = static_cast<double>(t.g);
  const double subx = __ddiv_rn(__dadd_rn(static_cast<double>(sx), ud(r.x)), gd);
  const double suby = __ddiv_rn(__dadd_rn(static_cast<double>(sy), ud(r.y)), gd);
  ox = __dmul_rn(__dadd_rn(static_cast<double>(px), subx), t.pw);
  oy = __dmul_rn(__dadd_rn(static_cast<double>(py), suby), t.ph);
}

__device__ __forceinline__ Crystal64 load64_parts(const ScanTile& t, uint32_t s) {
  Crystal64 k;
  const float4 d = t.d[s];
  k.morph = morph_of(d);
  if (t.pos64) {
    k.pos = d3(t.pos64[3 * s], t.pos64[3 * s + 1], t.pos64[3 * s + 2]);
    k.dims = d3(t.dims64[3 * s], t.dims64[3 * s + 1], t.dims64[3 * s + 2]);
#pragma unroll
    for (int j = 0; j < 4; ++j) k.q[j] = t.quat64[4 * s + j];
  } else {
    const float4 a = t.a[s], q = t.q[s];
    k.pos = d3(a.x, a.y, a.z);
    k.dims = d3(d.x, d.y, d.z);
    k.q[0] = q.x; k.q[1] = q.y; k.q[2] = q.z; k.q[3] = q.w;
  }
  k.sens = 1.0;
  return k;
}

// Exact FP64 chord of a vertical scan ray through crystal s (0 when it misses): the reference's
// geometry with the crystal's expansion, and the ray inside the box of the crystal's leaf.
static __device__ __noinline__ double scan_chord64(const ScanTile& t, uint32_t s, double ox, double oy,
                                            bool& hit) {
  const Crystal64 k = load64_parts(t, s);
  const double e = t.exp64[s];
  const D3 o = d3(ox, oy, t.z0);
  const D3 dir = d3(0.0, 0.0, -1.0);
  const D3 inv = d3(__ddiv_rn(1.0, 0.0), __ddiv_rn(1.0, 0.0), -1.0);
  double t0, t1;
  hit = rt_box_hit64(t.lbox64 + 6ull * t.leafof[s], o, inv) && dintersect(k, e, o, dir, t0, t1);
  return hit ? fmax(__dsub_rn(t1, t0), 0.0) : 0.0;
}

}  // namespace fg
