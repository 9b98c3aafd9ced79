// Fast-approximation mode: the reference's wgpu tile model (the compute shaders that
// GpuEngine::render_tile_all_gpu dispatches, gpu.rs:491-938) as CUDA kernels over many tiles at
// once.  It is a different model from the CPU path: one jittered crystal per grid cell
// (poisson.wgsl:62-133) relaxed once against its 26 neighbours (:135-190), a per-crystal Poisson
// photon count from the local pixel instead of photon transport (develop.wgsl:69-137), a
// clumping boost from developed neighbours (:139-202), and a scan of the 5 x 5 cell columns
// around each ray (scan.wgsl:55-178).  The Gaussian passes are not run: render_tile_all_gpu reads
// back the scan's density buffer (gpu.rs:912).
//
// Arithmetic is f32 in the shaders' operation order with every operation rounded on its own
// (intrinsics, no contraction).  Where WGSL leaves a choice to the implementation the same choice
// is made as in the CPU restatement: exp, log, sin and cos are evaluated in FP64 and rounded once;
// dot products sum (x + y) + z; the relaxation reads the positions from before its pass (the
// shader updates them in place, in an order the API leaves undefined).
//
// Layout: the grid cells of all tiles, 64 B each (position, dims and expansion, quaternion,
// flags), tile after tile; one launch per shader with blockIdx.y naming the tile.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fg_internal.h"

namespace fg {

namespace {

struct __align__(16) FastCell {
  float4 pos;       // xyz position (um)
  float4 dims_exp;  // xyz half-dimensions, w expansion
  float4 rot;       // quaternion
  uint4 flags;      // occupied, morphology, developed, absorbed photons
};
static_assert(sizeof(FastCell) == 64, "grid cell layout");

struct FastTile {
  unsigned long long cell_base, px_base, col_base;  // col_base: first (x, y) column of the tile
  const float* tile;  // exposure, width x height
  uint32_t gw, gh, gd, W, H, g;  // grid, pixels, strata per axis
  float cs, film_w, film_h, film_d, r_min, log_mean_r, var, ar, sens, exposure, fexp, clump, opacity;
  uint32_t morph, seed, scan_seed;
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fexp_(float x) { return static_cast<float>(exp(static_cast<double>(x))); }
__device__ __forceinline__ float flog_(float x) { return static_cast<float>(log(static_cast<double>(x))); }
__device__ __forceinline__ float fsin_(float x) { return static_cast<float>(sin(static_cast<double>(x))); }
__device__ __forceinline__ float fcos_(float x) { return static_cast<float>(cos(static_cast<double>(x))); }
__device__ __forceinline__ float clampf_(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ float dot3_(float ax, float ay, float az, float bx, float by, float bz) {
  return fa(fa(fm(ax, bx), fm(ay, by)), fm(az, bz));
}

constexpr float PI_F = 3.141592653589793f;

__device__ __forceinline__ uint32_t hash_u32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ float rand_f32(uint32_t& s) {
  s = hash_u32(s);
  return fd(__uint2float_rn(s), 4294967296.0f);
}

// Cell (x, y, z) of the tile for flat index i, false past the end.
__device__ __forceinline__ bool cell_xyz(const FastTile& t, unsigned long long i, uint32_t& x, uint32_t& y,
                                         uint32_t& z) {
  const unsigned long long n = static_cast<unsigned long long>(t.gw) * t.gh * t.gd;
  if (i >= n) return false;
  x = static_cast<uint32_t>(i % t.gw);
  y = static_cast<uint32_t>((i / t.gw) % t.gh);
  z = static_cast<uint32_t>(i / (static_cast<unsigned long long>(t.gw) * t.gh));
  return true;
}

// generate_candidates (poisson.wgsl:62-133); pos0 keeps the positions for the relaxation.
__global__ void k_fast_generate(const FastTile* __restrict__ tiles, FastCell* __restrict__ cells,
                                float4* __restrict__ pos0) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long n = static_cast<unsigned long long>(t.gw) * t.gh * t.gd;
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    uint32_t x, y, z;
    cell_xyz(t, i, x, y, z);
    uint32_t rng = t.seed ^ (x * 1973u + y * 9277u * 65537u + z * 26699u + 0x9E3779B9u);
    const float ox = fa(0.05f, fm(0.90f, rand_f32(rng)));
    const float oy = fa(0.05f, fm(0.90f, rand_f32(rng)));
    const float oz = fa(0.05f, fm(0.90f, rand_f32(rng)));
    FastCell c;
    c.pos = make_float4(clampf_(fm(fa(static_cast<float>(x), ox), t.cs), 0.0f, t.film_w),
                        clampf_(fm(fa(static_cast<float>(y), oy), t.cs), 0.0f, t.film_h),
                        clampf_(fm(fa(static_cast<float>(z), oz), t.cs), 0.0f, t.film_d), 0.0f);
    const float u1 = fmaxf(rand_f32(rng), 1e-6f);
    const float u2 = rand_f32(rng);
    const float nz = fm(__fsqrt_rn(fm(-2.0f, flog_(u1))), fcos_(fm(fm(2.0f, PI_F), u2)));
    const float radius = clampf_(fexp_(fa(t.log_mean_r, fm(t.var, nz))), 0.15f, fm(t.cs, 0.65f));
    if (t.morph == 1u) {
      const float aspect = fmaxf(t.ar, 1.0f);
      const float rp = fm(radius, __fsqrt_rn(aspect)), rt = fd(radius, __fsqrt_rn(aspect));
      c.dims_exp = make_float4(rp, rp, rt, 0.0f);
      const float tilt = fm(rand_f32(rng), 0.20f);
      const float phi = fm(fm(rand_f32(rng), 2.0f), PI_F);
      const float half = fm(tilt, 0.5f);
      c.rot = make_float4(fm(fsin_(half), fcos_(phi)), fm(fsin_(half), fsin_(phi)), 0.0f, fcos_(half));
    } else {
      c.dims_exp = make_float4(radius, radius, radius, 0.0f);
      const float q1 = rand_f32(rng), q2 = rand_f32(rng), q3 = rand_f32(rng);
      const float a2 = fm(fm(2.0f, PI_F), q2), a3 = fm(fm(2.0f, PI_F), q3);
      c.rot = make_float4(fm(__fsqrt_rn(fs(1.0f, q1)), fsin_(a2)), fm(__fsqrt_rn(fs(1.0f, q1)), fcos_(a2)),
                          fm(__fsqrt_rn(q1), fsin_(a3)), fm(__fsqrt_rn(q1), fcos_(a3)));
    }
    c.flags = make_uint4(1u, t.morph, 0u, 0u);
    cells[t.cell_base + i] = c;
    pos0[t.cell_base + i] = c.pos;
  }
}

// resolve_conflicts (poisson.wgsl:135-190) against the positions from before the pass.
__global__ void k_fast_resolve(const FastTile* __restrict__ tiles, FastCell* __restrict__ cells,
                               const float4* __restrict__ pos0) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long n = static_cast<unsigned long long>(t.gw) * t.gh * t.gd;
  const float4* P = pos0 + t.cell_base;
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    uint32_t x, y, z;
    cell_xyz(t, i, x, y, z);
    const float4 my = P[i];
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
    for (int dz = -1; dz <= 1; ++dz) {
      const int nz = static_cast<int>(z) + dz;
      if (nz < 0 || nz >= static_cast<int>(t.gd)) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int ny = static_cast<int>(y) + dy;
        if (ny < 0 || ny >= static_cast<int>(t.gh)) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int nx = static_cast<int>(x) + dx;
          if (nx < 0 || nx >= static_cast<int>(t.gw)) continue;
          if (dx == 0 && dy == 0 && dz == 0) continue;
          const float4 nb = P[(static_cast<unsigned long long>(nz) * t.gh + ny) * t.gw + nx];
          const float d0 = fs(my.x, nb.x), d1 = fs(my.y, nb.y), d2 = fs(my.z, nb.z);
          const float dd = dot3_(d0, d1, d2, d0, d1, d2);
          if (dd < fm(t.r_min, t.r_min) && dd > 1e-6f) {
            const float dist = __fsqrt_rn(dd);
            const float push = fd(fs(t.r_min, dist), dist);
            f0 = fa(f0, fm(d0, push));
            f1 = fa(f1, fm(d1, push));
            f2 = fa(f2, fm(d2, push));
          }
        }
      }
    }
    cells[t.cell_base + i].pos =
        make_float4(clampf_(fa(my.x, fm(f0, 0.25f)), 0.0f, t.film_w), clampf_(fa(my.y, fm(f1, 0.25f)), 0.0f, t.film_h),
                    clampf_(fa(my.z, fm(f2, 0.25f)), 0.0f, t.film_d), 0.0f);
  }
}

// develop.wgsl stage 0 (:69-137): Poisson photon count from the local pixel, dynamic threshold.
__global__ void k_fast_expose(const FastTile* __restrict__ tiles, FastCell* __restrict__ cells) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long n = static_cast<unsigned long long>(t.gw) * t.gh * t.gd;
  const float area_norm = static_cast<float>(0.55 * 0.55);  // an abstract-float constant, folded exactly
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    uint32_t x, y, z;
    cell_xyz(t, i, x, y, z);
    FastCell c = cells[t.cell_base + i];
    if (c.flags.x == 0u) continue;
    const float u = clampf_(fd(c.pos.x, t.film_w), 0.0f, 1.0f), v = clampf_(fd(c.pos.y, t.film_h), 0.0f, 1.0f);
    const uint32_t px = min(static_cast<uint32_t>(rintf(fm(u, static_cast<float>(t.W - 1u)))), t.W - 1u);
    const uint32_t py = min(static_cast<uint32_t>(rintf(fm(v, static_cast<float>(t.H - 1u)))), t.H - 1u);
    const float irr = fm(t.tile[static_cast<size_t>(py) * t.W + px], t.exposure);
    if (irr < 0.05f) {
      c.flags.z = 0u;
      c.dims_exp.w = 0.0f;
      c.flags.x = 0u;
      cells[t.cell_base + i] = c;
      continue;
    }
    const float att = fexp_(fm(-0.10f, c.pos.z));
    const float radius = c.dims_exp.x;
    const float area = fd(fm(radius, radius), area_norm);
    const float expected = fm(fm(fm(fm(irr, att), area), t.sens), 1.6f);
    uint32_t rng = t.seed ^ (x * 1973u + y * 9277u * 65537u + z * 26699u + 0x85EBCA6Bu);
    const float L = fexp_(-fminf(expected, 30.0f));
    uint32_t k = 0;
    float p = 1.0f;
    while (p > L && k < 40u) {  // at most 40 draws
      k = k + 1u;
      p = fm(p, rand_f32(rng));
    }
    uint32_t absorbed = k > 0u ? k - 1u : 0u;
    if (expected > 30.0f) {
      const float u1 = fmaxf(rand_f32(rng), 1e-6f);
      const float u2 = rand_f32(rng);
      const float nz = fm(__fsqrt_rn(fm(-2.0f, flog_(u1))), fcos_(fm(fm(2.0f, PI_F), u2)));
      const float approx = fa(expected, fm(__fsqrt_rn(expected), nz));
      absorbed = static_cast<uint32_t>(fmaxf(approx, 0.0f));
    }
    c.flags.w = absorbed;
    const float speck = rand_f32(rng);
    const float base_t = speck < 0.30f ? 3.0f : 4.0f;
    const float ratio = clampf_(fd(0.55f, fmaxf(radius, 0.20f)), 0.75f, 1.8f);
    const uint32_t thr = static_cast<uint32_t>(fmaxf(rintf(fm(base_t, ratio)), 2.0f));
    if (absorbed >= thr) {
      c.flags.z = 1u;
      c.dims_exp.w = t.fexp;
    } else {
      c.flags.z = 0u;
      c.dims_exp.w = 0.0f;
      c.flags.x = 0u;
    }
    cells[t.cell_base + i] = c;
  }
}

// develop.wgsl stage 1 (:139-202): the neighbours' flags and positions do not change in this pass,
// so the in-place update of the expansion is deterministic.
__global__ void k_fast_clump(const FastTile* __restrict__ tiles, FastCell* __restrict__ cells) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long n = static_cast<unsigned long long>(t.gw) * t.gh * t.gd;
  FastCell* C = cells + t.cell_base;
  const float reach = fm(fm(t.cs, t.clump), 1.50f);
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    uint32_t x, y, z;
    cell_xyz(t, i, x, y, z);
    const uint4 fl = C[i].flags;
    if (fl.x == 0u || fl.z == 0u) continue;
    const float4 cp = C[i].pos;
    uint32_t touching = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      const int nz = static_cast<int>(z) + dz;
      if (nz < 0 || nz >= static_cast<int>(t.gd)) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int ny = static_cast<int>(y) + dy;
        if (ny < 0 || ny >= static_cast<int>(t.gh)) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int nx = static_cast<int>(x) + dx;
          if (nx < 0 || nx >= static_cast<int>(t.gw)) continue;
          if (dx == 0 && dy == 0 && dz == 0) continue;
          const size_t j = (static_cast<size_t>(nz) * t.gh + ny) * t.gw + nx;
          const uint4 nf = C[j].flags;
          if (nf.x == 1u && nf.z == 1u) {
            const float4 np = C[j].pos;
            const float d0 = fs(np.x, cp.x), d1 = fs(np.y, cp.y), d2 = fs(np.z, cp.z);
            if (dot3_(d0, d1, d2, d0, d1, d2) <= fm(reach, reach)) ++touching;
          }
        }
      }
    }
    if (touching > 0u)
      C[i].dims_exp.w = fm(C[i].dims_exp.w, fa(1.15f, fm(0.12f, static_cast<float>(min(touching, 12u)))));
  }
}

// Bitmask over depth of the developed crystals of each (x, y) column (the grid is at most 32 deep),
// so the scan visits developed cells only, in the same depth order.
__global__ void k_fast_colmask(const FastTile* __restrict__ tiles, const FastCell* __restrict__ cells,
                               uint32_t* __restrict__ colmask) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long ncol = static_cast<unsigned long long>(t.gw) * t.gh;
  const FastCell* C = cells + t.cell_base;
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < ncol;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    uint32_t m = 0;
    for (uint32_t z = 0; z < t.gd; ++z) {
      const uint4 fl = C[static_cast<size_t>(z) * ncol + i].flags;
      if (fl.x != 0u && fl.z != 0u) m |= 1u << z;
    }
    colmask[t.col_base + i] = m;
  }
}

__device__ __forceinline__ void cross3(float ax, float ay, float az, float bx, float by, float bz, float& ox, float& oy,
                                       float& oz) {
  ox = fs(fm(ay, bz), fm(az, by));
  oy = fs(fm(az, bx), fm(ax, bz));
  oz = fs(fm(ax, by), fm(ay, bx));
}

__device__ __forceinline__ void quat_inv_rot(float4 q, float vx, float vy, float vz, float& ox, float& oy,
                                             float& oz) {
  const float qx = -q.x, qy = -q.y, qz = -q.z;
  float cx, cy, cz;
  cross3(qx, qy, qz, vx, vy, vz, cx, cy, cz);
  const float tx = fm(2.0f, cx), ty = fm(2.0f, cy), tz = fm(2.0f, cz);
  float c2x, c2y, c2z;
  cross3(qx, qy, qz, tx, ty, tz, c2x, c2y, c2z);
  ox = fa(fa(vx, fm(q.w, tx)), c2x);
  oy = fa(fa(vy, fm(q.w, ty)), c2y);
  oz = fa(fa(vz, fm(q.w, tz)), c2z);
}

// scan.wgsl:55-178: per pixel, g x g jittered vertical rays through the 5 x 5 cell columns.
__global__ void k_fast_scan(const FastTile* __restrict__ tiles, const FastCell* __restrict__ cells,
                            const uint32_t* __restrict__ colmask, float* __restrict__ d_neg) {
  const FastTile t = tiles[blockIdx.y];
  const unsigned long long npx = static_cast<unsigned long long>(t.W) * t.H;
  const FastCell* C = cells + t.cell_base;
  const float pw = fd(t.film_w, static_cast<float>(t.W)), ph = fd(t.film_h, static_cast<float>(t.H));
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < npx;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const uint32_t px = static_cast<uint32_t>(i % t.W), py = static_cast<uint32_t>(i / t.W);
    uint32_t rng = t.scan_seed ^ (px * 1973u + py * 9277u * 65537u + 1013904223u);
    float acc = 0.0f;
    for (uint32_t sy = 0; sy < t.g; ++sy)
      for (uint32_t sx = 0; sx < t.g; ++sx) {
        const float sub_x = fd(fa(static_cast<float>(sx), rand_f32(rng)), static_cast<float>(t.g));
        const float sub_y = fd(fa(static_cast<float>(sy), rand_f32(rng)), static_cast<float>(t.g));
        const float ox = fm(fa(static_cast<float>(px), sub_x), pw);
        const float oy = fm(fa(static_cast<float>(py), sub_y), ph);
        const float oz = fa(t.film_d, 0.1f);
        float total = 0.0f;
        const int cx = static_cast<int>(floorf(fd(ox, t.cs))), cy = static_cast<int>(floorf(fd(oy, t.cs)));
        for (int dy = -2; dy <= 2; ++dy) {
          const int gy = cy + dy;
          if (gy < 0 || gy >= static_cast<int>(t.gh)) continue;
          for (int dx = -2; dx <= 2; ++dx) {
            const int gx = cx + dx;
            if (gx < 0 || gx >= static_cast<int>(t.gw)) continue;
            for (uint32_t m = __ldg(colmask + t.col_base + static_cast<size_t>(gy) * t.gw + gx); m; m &= m - 1) {
              const int gz = __ffs(m) - 1;
              const FastCell* c = C + (static_cast<size_t>(gz) * t.gh + gy) * t.gw + gx;
              const uint4 fl = __ldg(&c->flags);
              const float4 cp = __ldg(&c->pos), de = __ldg(&c->dims_exp), q = __ldg(&c->rot);
              float lox, loy, loz, ldx, ldy, ldz;
              quat_inv_rot(q, fs(ox, cp.x), fs(oy, cp.y), fs(oz, cp.z), lox, loy, loz);
              quat_inv_rot(q, 0.0f, 0.0f, -1.0f, ldx, ldy, ldz);
              const float dmx = fm(de.x, de.w), dmy = fm(de.y, de.w), dmz = fm(de.z, de.w);
              if (fl.y == 0u) {
                auto axis = [](float ld, float lo, float dm, float& tmin, float& tmax) {
                  const float sgn = ld > 0.0f ? 1.0f : (ld < 0.0f ? -1.0f : 0.0f);
                  const float safe_sign = sgn == 0.0f ? 1.0f : sgn;
                  const float sd = fabsf(ld) < 1e-6f ? fm(safe_sign, 1e-6f) : ld;
                  const float inv = fd(1.0f, sd);
                  const float t1 = fm(fs(-dm, lo), inv), t2 = fm(fs(dm, lo), inv);
                  tmin = fminf(t1, t2);
                  tmax = fmaxf(t1, t2);
                };
                float a0, b0, a1, b1, a2, b2;
                axis(ldx, lox, dmx, a0, b0);
                axis(ldy, loy, dmy, a1, b1);
                axis(ldz, loz, dmz, a2, b2);
                const float te = fmaxf(fmaxf(a0, a1), a2), tx = fminf(fminf(b0, b1), b2);
                if (tx >= te && tx > 0.0f) {
                  const float path = fs(tx, fmaxf(te, 0.0f));
                  if (path > 0.0f) total = fa(total, path);
                }
              } else {
                const float p0 = fd(lox, dmx), p1 = fd(loy, dmy), p2 = fd(loz, dmz);
                const float e0 = fd(ldx, dmx), e1 = fd(ldy, dmy), e2 = fd(ldz, dmz);
                const float a = dot3_(e0, e1, e2, e0, e1, e2);
                if (a > 1e-6f) {
                  const float b = fm(2.0f, dot3_(p0, p1, p2, e0, e1, e2));
                  const float cc = fs(dot3_(p0, p1, p2, p0, p1, p2), 1.0f);
                  const float disc = fs(fm(b, b), fm(fm(4.0f, a), cc));
                  if (disc >= 0.0f) {
                    const float sq = __fsqrt_rn(disc);
                    const float inv2a = fd(0.5f, a);
                    const float t0 = fm(fs(-b, sq), inv2a), t1 = fm(fa(-b, sq), inv2a);
                    const float te = fminf(t0, t1), tx = fmaxf(t0, t1);
                    if (tx > 0.0f && tx >= te) {
                      const float path = fs(tx, fmaxf(te, 0.0f));
                      if (path > 0.0f) total = fa(total, path);
                    }
                  }
                }
              }
            }
          }
        }
        const float safe = clampf_(total, 0.0f, t.film_d);
        acc = fa(acc, fexp_(fm(-t.opacity, safe)));
      }
    const float mean_t = clampf_(fd(acc, static_cast<float>(t.g * t.g)), 1e-4f, 1.0f);
    d_neg[t.px_base + i] = fa(fd(-flog_(mean_t), 2.302585092994046f), 0.05f);
  }
}

// The cell grid of a tile (gpu.rs:505-525): cells of max(r_min, 1) um, at most 512 per side in
// the plane (the cell grows when the tile is larger) and 32 in depth.
void fast_grid(const fg_tile_params& p, uint32_t& gw, uint32_t& gh, uint32_t& gd, float& cs) {
  cs = static_cast<float>(std::max(p.r_min, 1.0));
  const uint32_t maxd = 512;
  const uint32_t rw = static_cast<uint32_t>(std::ceil(static_cast<float>(p.film_w) / cs));
  const uint32_t rh = static_cast<uint32_t>(std::ceil(static_cast<float>(p.film_h) / cs));
  if (rw > maxd || rh > maxd) {
    const float scale = static_cast<float>(std::max(rw, rh)) / static_cast<float>(maxd);
    cs = cs * scale;
    gw = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p.film_w) / cs)), 1u), maxd);
    gh = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p.film_h) / cs)), 1u), maxd);
  } else {
    gw = std::max(rw, 1u);
    gh = std::max(rh, 1u);
  }
  gd = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p.film_d) / cs)), 1u), 32u);
}

FastTile fast_tile(const fg_tile_params& p) {
  FastTile t{};
  fast_grid(p, t.gw, t.gh, t.gd, t.cs);
  t.W = p.width_px;
  t.H = p.height_px;
  const uint32_t spp = std::max(p.samples_per_pixel, 1u);
  t.g = std::max(static_cast<uint32_t>(std::nearbyint(std::sqrt(static_cast<float>(spp)))), 1u);
  t.film_w = static_cast<float>(p.film_w);
  t.film_h = static_cast<float>(p.film_h);
  t.film_d = static_cast<float>(p.film_d);
  t.r_min = static_cast<float>(p.r_min);
  // log(mean radius) once per tile, in double and rounded once, as every cell would form it.
  t.log_mean_r = static_cast<float>(std::log(static_cast<double>(static_cast<float>(p.mean_crystal_radius))));
  t.var = static_cast<float>(p.size_variance);
  t.ar = static_cast<float>(p.tabular_aspect_ratio);
  t.sens = static_cast<float>(p.base_sensitivity);
  t.exposure = static_cast<float>(p.exposure);
  t.fexp = static_cast<float>(p.filament_expansion);
  t.clump = static_cast<float>(p.clumping_proximity_factor);
  t.opacity = static_cast<float>(p.silver_opacity);
  t.morph = static_cast<uint32_t>(p.morphology);
  t.seed = static_cast<uint32_t>(p.seed & 0xffffffffu);
  t.scan_seed = static_cast<uint32_t>((p.seed + 1013904223ull) & 0xffffffffu);  // gpu.rs:732
  return t;
}

}  // namespace

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_fast_grid(const fg_tile_params* p, uint32_t* dims, float* cell_size) {
  if (!p || !dims) return FG_ERR_INVALID_ARG;
  float cs;
  fast_grid(*p, dims[0], dims[1], dims[2], cs);
  if (cell_size) *cell_size = cs;
  return FG_OK;
}

fg_status fg_render_tiles_fast(fg_engine* e, const fg_tile_params* params, uint32_t ntiles, const float* const* tiles,
                               float* const* d_neg, void* const* cells) {
  return guard(e, [&] {
    FG_REQUIRE(params && tiles && d_neg && ntiles > 0 && ntiles <= 65535, "null argument or bad tile count");
    cudaStream_t st = e->stream;
    std::vector<FastTile> ft(ntiles);
    unsigned long long nc = 0, npx = 0, maxc = 0, maxp = 0, ncols = 0;
    for (uint32_t i = 0; i < ntiles; ++i) {
      const fg_tile_params& p = params[i];
      FG_REQUIRE(tiles[i] && d_neg[i], "null tile or output");
      FG_REQUIRE(p.width_px > 0 && p.height_px > 0, "empty tile");
      FG_REQUIRE(p.film_w > 0 && p.film_h > 0 && p.film_d > 0 && p.r_min > 0, "bad film geometry");
      FG_REQUIRE(p.morphology >= 0 && p.morphology <= 2, "morphology out of range");
      ft[i] = fast_tile(p);
      ft[i].cell_base = nc;
      ft[i].px_base = npx;
      ft[i].col_base = ncols;
      ncols += static_cast<unsigned long long>(ft[i].gw) * ft[i].gh;
      const unsigned long long c = static_cast<unsigned long long>(ft[i].gw) * ft[i].gh * ft[i].gd;
      const unsigned long long q = static_cast<unsigned long long>(p.width_px) * p.height_px;
      nc += c;
      npx += q;
      maxc = std::max(maxc, c);
      maxp = std::max(maxp, q);
    }
    DBuf<float> img(npx, st), out(npx, st);
    DBuf<FastCell> dc(nc, st);
    DBuf<float4> pos0(nc, st);
    DBuf<uint32_t> colmask(ncols, st);
    for (uint32_t i = 0; i < ntiles; ++i) {
      ft[i].tile = img.p + ft[i].px_base;
      FG_CUDA(cudaMemcpyAsync(img.p + ft[i].px_base, tiles[i],
                              static_cast<size_t>(params[i].width_px) * params[i].height_px * sizeof(float),
                              cudaMemcpyHostToDevice, st));
    }
    DBuf<FastTile> dt(ntiles, st);
    FG_CUDA(cudaMemcpyAsync(dt.p, ft.data(), ntiles * sizeof(FastTile), cudaMemcpyHostToDevice, st));
    const unsigned bc = static_cast<unsigned>(std::min<unsigned long long>(grid_for(maxc, 256), 4096));
    const unsigned bp = static_cast<unsigned>(std::min<unsigned long long>(grid_for(maxp, 128), 4096));
    k_fast_generate<<<dim3(bc, ntiles), 256, 0, st>>>(dt.p, dc.p, pos0.p);
    k_fast_resolve<<<dim3(bc, ntiles), 256, 0, st>>>(dt.p, dc.p, pos0.p);
    k_fast_expose<<<dim3(bc, ntiles), 256, 0, st>>>(dt.p, dc.p);
    k_fast_clump<<<dim3(bc, ntiles), 256, 0, st>>>(dt.p, dc.p);
    k_fast_colmask<<<dim3(bc, ntiles), 256, 0, st>>>(dt.p, dc.p, colmask.p);
    k_fast_scan<<<dim3(bp, ntiles), 128, 0, st>>>(dt.p, dc.p, colmask.p, out.p);
    FG_CUDA(cudaGetLastError());
    for (uint32_t i = 0; i < ntiles; ++i) {
      FG_CUDA(cudaMemcpyAsync(d_neg[i], out.p + ft[i].px_base,
                              static_cast<size_t>(params[i].width_px) * params[i].height_px * sizeof(float),
                              cudaMemcpyDeviceToHost, st));
      if (cells && cells[i])
        FG_CUDA(cudaMemcpyAsync(cells[i], dc.p + ft[i].cell_base,
                                static_cast<size_t>(ft[i].gw) * ft[i].gh * ft[i].gd * sizeof(FastCell),
                                cudaMemcpyDeviceToHost, st));
    }
    FG_CUDA(cudaStreamSynchronize(st));
  });
}

fg_status fg_render_tile_fast(fg_engine* e, const float* tile, const fg_tile_params* p, float* d_neg, void* cells) {
  if (!p) return FG_ERR_INVALID_ARG;
  return fg_render_tiles_fast(e, p, 1, &tile, &d_neg, cells ? &cells : nullptr);
}

// GpuTileParams of the reference's GPU branch (image_pipeline.rs:455-518): the preset alone picks
// the stock (no switch to the 1600 emulsion at push >= 1.5, unlike the CPU tile worker).
fg_status fg_tile_params_fast_preset(const char* preset, double pixel_size_um, uint32_t tw, uint32_t th,
                                     double exposure, double push, uint64_t tile_seed, fg_tile_params* out) {
  if (!preset || !out || !(pixel_size_um > 0) || tw == 0 || th == 0) return FG_ERR_INVALID_ARG;
  std::string s(preset);
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  const bool tmax = s == "t-max" || s == "tmax", hp5 = s == "hp5" || s == "hp5-plus";
  const bool x1600 = s == "tri-x-1600" || s == "trix-1600" || s == "caffenol";
  const double eff_push = (s.find("1600") != std::string::npos || s == "caffenol") ? std::max(push, 2.0)
                                                                                   : std::max(push, 0.0);
  *out = fg_tile_params{};
  out->film_w = tw * pixel_size_um;
  out->film_h = th * pixel_size_um;
  out->film_d = tmax ? 8.0 : (hp5 ? 12.5 : (x1600 ? 14.5 : 14.0));
  out->width_px = tw;
  out->height_px = th;
  out->samples_per_pixel = 4;
  out->silver_opacity = tmax ? 0.18 : (hp5 ? 0.22 : 0.25);
  out->seed = tile_seed;
  out->r_min = tmax ? 0.9 : (hp5 ? 1.1 : (x1600 ? 1.1 : 1.2));
  out->mean_crystal_radius = tmax ? 0.40 : (hp5 ? 0.50 : (x1600 ? 0.52 : 0.55));
  out->size_variance = tmax ? 0.20 : (hp5 ? 0.30 : (x1600 ? 0.38 : 0.40));
  out->morphology = tmax ? 1 : (hp5 ? 2 : 0);
  out->tabular_aspect_ratio = 6.5;
  out->base_sensitivity = tmax ? 0.8 : (hp5 ? 1.1 : (x1600 ? 1.35 : 1.2));
  out->exposure = exposure;
  out->threshold_photons = 4;
  out->filament_expansion = tmax ? 1.10 + 0.04 * eff_push : (hp5 ? 1.15 + 0.05 * eff_push : 1.20 + 0.06 * eff_push);
  out->clumping_proximity_factor =
      tmax ? 1.10 + 0.03 * eff_push : (hp5 ? 1.18 + 0.04 * eff_push : 1.25 + 0.05 * eff_push);
  return FG_OK;
}

}  // extern "C"
