// CPU oracle of the reference's wgpu tile model (TEST INFRASTRUCTURE ONLY: the tests use it as
// the checker of the CUDA library's fast-approximation mode; the product never links it).
//
// Restates the compute shaders that GpuEngine::render_tile_all_gpu dispatches (gpu.rs:491-938):
//   poisson.wgsl:62-133   generate_candidates: one jittered crystal per grid cell
//   poisson.wgsl:135-190  resolve_conflicts: one relaxation step against the 26 neighbours
//   develop.wgsl:69-137   stage 0: per-crystal Poisson photon count from the local pixel, dynamic
//                         threshold, shadow cut
//   develop.wgsl:139-202  stage 1: clumping boost from the developed neighbours
//   scan.wgsl:55-178      per-pixel jittered rays through the 5 x 5 cell columns
// and the grid set-up of gpu.rs:505-525.  The Gaussian passes (gaussian.wgsl) are not restated:
// render_tile_all_gpu reads back the scan's density buffer (gpu.rs:912), not their output.
//
// Arithmetic is f32 in the shaders' operation order, without contraction.  Where WGSL leaves a
// choice to the implementation, this restatement (and the device) fix it:
//   * exp, log, sin and cos are evaluated in double and rounded once to float;
//   * dot(a, b) sums (a.x b.x + a.y b.y) + a.z b.z;
//   * resolve_conflicts reads the positions from before the pass (the shader updates them in
//     place, so an invocation may see some neighbours already moved, in an order the API leaves
//     undefined);
//   * constant expressions of abstract floats (0.55 * 0.55) are folded in double, then rounded.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fg_oracle.h"

namespace {

struct Cell {
  float pos[4], dims_exp[4], rot[4];
  uint32_t flags[4];
};
static_assert(sizeof(Cell) == 64, "grid cell layout");

constexpr float PI_F = 3.141592653589793f;

uint32_t hash_u32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

float rand_f32(uint32_t& s) {
  s = hash_u32(s);
  return static_cast<float>(s) / 4294967296.0f;
}

float fexp(float x) { return static_cast<float>(std::exp(static_cast<double>(x))); }
float flog(float x) { return static_cast<float>(std::log(static_cast<double>(x))); }
float fsin(float x) { return static_cast<float>(std::sin(static_cast<double>(x))); }
float fcos(float x) { return static_cast<float>(std::cos(static_cast<double>(x))); }
float clampf(float v, float lo, float hi) { return std::fmin(std::fmax(v, lo), hi); }
float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

void cross3(const float* a, const float* b, float* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

void quat_inv_rot(const float* q, const float* v, float* out) {
  const float qv[3] = {-q[0], -q[1], -q[2]};
  float c[3], t[3], c2[3];
  cross3(qv, v, c);
  for (int k = 0; k < 3; ++k) t[k] = 2.0f * c[k];
  cross3(qv, t, c2);
  for (int k = 0; k < 3; ++k) out[k] = (v[k] + q[3] * t[k]) + c2[k];
}

}  // namespace

extern "C" {

int or_fast_grid(const or_fast_params* p, or_fast_grid_t* g) {
  float cs = static_cast<float>(std::max(p->r_min, 1.0));
  const uint32_t maxd = 512;
  const uint32_t rw = static_cast<uint32_t>(std::ceil(static_cast<float>(p->film_w) / cs));
  const uint32_t rh = static_cast<uint32_t>(std::ceil(static_cast<float>(p->film_h) / cs));
  uint32_t gw, gh;
  if (rw > maxd || rh > maxd) {
    const float scale = static_cast<float>(std::max(rw, rh)) / static_cast<float>(maxd);
    cs = cs * scale;
    gw = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p->film_w) / cs)), 1u), maxd);
    gh = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p->film_h) / cs)), 1u), maxd);
  } else {
    gw = std::max(rw, 1u);
    gh = std::max(rh, 1u);
  }
  const uint32_t gd = std::min(std::max(static_cast<uint32_t>(std::ceil(static_cast<float>(p->film_d) / cs)), 1u), 32u);
  g->w = gw;
  g->h = gh;
  g->d = gd;
  g->cell_size = cs;
  return 0;
}

int or_fast_tile(const or_fast_params* p, const float* tile, float* d_neg, void* cells_out) {
  or_fast_grid_t G;
  or_fast_grid(p, &G);
  const uint32_t gw = G.w, gh = G.h, gd = G.d;
  const float cs = G.cell_size;
  const size_t nc = static_cast<size_t>(gw) * gh * gd;
  std::vector<Cell> cells(nc);
  const float film_w = static_cast<float>(p->film_w), film_h = static_cast<float>(p->film_h);
  const float film_d = static_cast<float>(p->film_d);
  const uint32_t seed = static_cast<uint32_t>(p->seed & 0xffffffffu);
  // generate_candidates (poisson.wgsl:62-133).
  const float mean_r = static_cast<float>(p->mean_crystal_radius), var = static_cast<float>(p->size_variance);
  const float ar = static_cast<float>(p->tabular_aspect_ratio);
  for (uint32_t z = 0; z < gd; ++z)
    for (uint32_t y = 0; y < gh; ++y)
      for (uint32_t x = 0; x < gw; ++x) {
        Cell& c = cells[(static_cast<size_t>(z) * gh + y) * gw + x];
        uint32_t rng = seed ^ (x * 1973u + y * 9277u * 65537u + z * 26699u + 0x9E3779B9u);
        const float ox = 0.05f + 0.90f * rand_f32(rng);
        const float oy = 0.05f + 0.90f * rand_f32(rng);
        const float oz = 0.05f + 0.90f * rand_f32(rng);
        c.pos[0] = clampf((static_cast<float>(x) + ox) * cs, 0.0f, film_w);
        c.pos[1] = clampf((static_cast<float>(y) + oy) * cs, 0.0f, film_h);
        c.pos[2] = clampf((static_cast<float>(z) + oz) * cs, 0.0f, film_d);
        c.pos[3] = 0.0f;
        const float u1 = std::fmax(rand_f32(rng), 1e-6f);
        const float u2 = rand_f32(rng);
        const float nz = std::sqrt(-2.0f * flog(u1)) * fcos((2.0f * PI_F) * u2);
        const float radius = clampf(fexp(flog(mean_r) + var * nz), 0.15f, cs * 0.65f);
        float dims[3] = {radius, radius, radius};
        float rot[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        if (p->morphology == 1) {
          const float aspect = std::fmax(ar, 1.0f);
          const float rp = radius * std::sqrt(aspect), rt = radius / std::sqrt(aspect);
          dims[0] = rp;
          dims[1] = rp;
          dims[2] = rt;
          const float tilt = rand_f32(rng) * 0.20f;
          const float phi = rand_f32(rng) * 2.0f * PI_F;
          const float half = tilt * 0.5f;
          rot[0] = fsin(half) * fcos(phi);
          rot[1] = fsin(half) * fsin(phi);
          rot[2] = 0.0f;
          rot[3] = fcos(half);
        } else {
          const float q1 = rand_f32(rng), q2 = rand_f32(rng), q3 = rand_f32(rng);
          rot[0] = std::sqrt(1.0f - q1) * fsin((2.0f * PI_F) * q2);
          rot[1] = std::sqrt(1.0f - q1) * fcos((2.0f * PI_F) * q2);
          rot[2] = std::sqrt(q1) * fsin((2.0f * PI_F) * q3);
          rot[3] = std::sqrt(q1) * fcos((2.0f * PI_F) * q3);
        }
        for (int k = 0; k < 3; ++k) c.dims_exp[k] = dims[k];
        c.dims_exp[3] = 0.0f;
        for (int k = 0; k < 4; ++k) c.rot[k] = rot[k];
        c.flags[0] = 1u;
        c.flags[1] = p->morphology;
        c.flags[2] = 0u;
        c.flags[3] = 0u;
      }
  // resolve_conflicts (poisson.wgsl:135-190), positions from before the pass.
  {
    std::vector<Cell> old(cells);
    const float rmin = static_cast<float>(p->r_min);
    for (uint32_t z = 0; z < gd; ++z)
      for (uint32_t y = 0; y < gh; ++y)
        for (uint32_t x = 0; x < gw; ++x) {
          const size_t ci = (static_cast<size_t>(z) * gh + y) * gw + x;
          const float* my = old[ci].pos;
          float f[3] = {0.0f, 0.0f, 0.0f};
          for (int dz = -1; dz <= 1; ++dz) {
            const int nz = static_cast<int>(z) + dz;
            if (nz < 0 || nz >= static_cast<int>(gd)) continue;
            for (int dy = -1; dy <= 1; ++dy) {
              const int ny = static_cast<int>(y) + dy;
              if (ny < 0 || ny >= static_cast<int>(gh)) continue;
              for (int dx = -1; dx <= 1; ++dx) {
                const int nx = static_cast<int>(x) + dx;
                if (nx < 0 || nx >= static_cast<int>(gw)) continue;
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const float* nb = old[(static_cast<size_t>(nz) * gh + ny) * gw + nx].pos;
                const float diff[3] = {my[0] - nb[0], my[1] - nb[1], my[2] - nb[2]};
                const float d2 = dot3(diff, diff);
                if (d2 < rmin * rmin && d2 > 1e-6f) {
                  const float dist = std::sqrt(d2);
                  const float push = (rmin - dist) / dist;
                  for (int k = 0; k < 3; ++k) f[k] = f[k] + diff[k] * push;
                }
              }
            }
          }
          cells[ci].pos[0] = clampf(my[0] + f[0] * 0.25f, 0.0f, film_w);
          cells[ci].pos[1] = clampf(my[1] + f[1] * 0.25f, 0.0f, film_h);
          cells[ci].pos[2] = clampf(my[2] + f[2] * 0.25f, 0.0f, film_d);
          cells[ci].pos[3] = 0.0f;
        }
  }
  // develop stage 0 (develop.wgsl:69-137).
  const uint32_t W = p->width_px, H = p->height_px;
  const float exposure = static_cast<float>(p->exposure), sens = static_cast<float>(p->base_sensitivity);
  const float fexp_v = static_cast<float>(p->filament_expansion);
  const float area_norm = static_cast<float>(0.55 * 0.55);
  for (uint32_t z = 0; z < gd; ++z)
    for (uint32_t y = 0; y < gh; ++y)
      for (uint32_t x = 0; x < gw; ++x) {
        Cell& c = cells[(static_cast<size_t>(z) * gh + y) * gw + x];
        if (c.flags[0] == 0u) continue;
        const float u = clampf(c.pos[0] / film_w, 0.0f, 1.0f), v = clampf(c.pos[1] / film_h, 0.0f, 1.0f);
        const uint32_t px = std::min(static_cast<uint32_t>(std::nearbyint(u * static_cast<float>(W - 1u))), W - 1u);
        const uint32_t py = std::min(static_cast<uint32_t>(std::nearbyint(v * static_cast<float>(H - 1u))), H - 1u);
        const float irr = tile[static_cast<size_t>(py) * W + px] * exposure;
        if (irr < 0.05f) {
          c.flags[2] = 0u;
          c.dims_exp[3] = 0.0f;
          c.flags[0] = 0u;
          continue;
        }
        const float att = fexp(-0.10f * c.pos[2]);
        const float radius = c.dims_exp[0];
        const float area = (radius * radius) / area_norm;
        const float expected = irr * att * area * sens * 1.6f;
        uint32_t rng = seed ^ (x * 1973u + y * 9277u * 65537u + z * 26699u + 0x85EBCA6Bu);
        const float L = fexp(-std::fmin(expected, 30.0f));
        uint32_t k = 0;
        float pr = 1.0f;
        while (pr > L && k < 40u) {
          k = k + 1u;
          pr = pr * rand_f32(rng);
        }
        uint32_t absorbed = k > 0u ? k - 1u : 0u;
        if (expected > 30.0f) {
          const float u1 = std::fmax(rand_f32(rng), 1e-6f);
          const float u2 = rand_f32(rng);
          const float nz = std::sqrt(-2.0f * flog(u1)) * fcos((2.0f * PI_F) * u2);
          const float approx = expected + std::sqrt(expected) * nz;
          absorbed = static_cast<uint32_t>(std::fmax(approx, 0.0f));
        }
        c.flags[3] = absorbed;
        const float speck = rand_f32(rng);
        const float base_t = speck < 0.30f ? 3.0f : 4.0f;
        const float ratio = clampf(0.55f / std::fmax(radius, 0.20f), 0.75f, 1.8f);
        const uint32_t thr = static_cast<uint32_t>(std::fmax(std::nearbyint(base_t * ratio), 2.0f));
        if (absorbed >= thr) {
          c.flags[2] = 1u;
          c.dims_exp[3] = fexp_v;
        } else {
          c.flags[2] = 0u;
          c.dims_exp[3] = 0.0f;
          c.flags[0] = 0u;
        }
      }
  // develop stage 1 (develop.wgsl:139-202): neighbours' flags and positions do not change here.
  {
    const float reach = cs * static_cast<float>(p->clumping_proximity_factor) * 1.50f;
    std::vector<float> boosted(nc, -1.0f);
    for (uint32_t z = 0; z < gd; ++z)
      for (uint32_t y = 0; y < gh; ++y)
        for (uint32_t x = 0; x < gw; ++x) {
          const size_t ci = (static_cast<size_t>(z) * gh + y) * gw + x;
          const Cell& c = cells[ci];
          if (c.flags[0] == 0u || c.flags[2] == 0u) continue;
          uint32_t touching = 0;
          for (int dz = -1; dz <= 1; ++dz) {
            const int nz = static_cast<int>(z) + dz;
            if (nz < 0 || nz >= static_cast<int>(gd)) continue;
            for (int dy = -1; dy <= 1; ++dy) {
              const int ny = static_cast<int>(y) + dy;
              if (ny < 0 || ny >= static_cast<int>(gh)) continue;
              for (int dx = -1; dx <= 1; ++dx) {
                const int nx = static_cast<int>(x) + dx;
                if (nx < 0 || nx >= static_cast<int>(gw)) continue;
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const Cell& nb = cells[(static_cast<size_t>(nz) * gh + ny) * gw + nx];
                if (nb.flags[0] == 1u && nb.flags[2] == 1u) {
                  const float diff[3] = {nb.pos[0] - c.pos[0], nb.pos[1] - c.pos[1], nb.pos[2] - c.pos[2]};
                  if (dot3(diff, diff) <= reach * reach) ++touching;
                }
              }
            }
          }
          if (touching > 0u)
            boosted[ci] = c.dims_exp[3] * (1.15f + 0.12f * static_cast<float>(std::min(touching, 12u)));
        }
    for (size_t i = 0; i < nc; ++i)
      if (boosted[i] >= 0.0f) cells[i].dims_exp[3] = boosted[i];
  }
  // scan (scan.wgsl:55-178).
  const uint32_t spp = std::max(p->samples_per_pixel, 1u);
  const uint32_t g = std::max(static_cast<uint32_t>(std::nearbyint(std::sqrt(static_cast<float>(spp)))), 1u);
  const float pw = film_w / static_cast<float>(W), ph = film_h / static_cast<float>(H);
  const uint32_t sseed = static_cast<uint32_t>((p->seed + 1013904223ull) & 0xffffffffu);
  const float opacity = static_cast<float>(p->silver_opacity);
  for (uint32_t py = 0; py < H; ++py)
    for (uint32_t px = 0; px < W; ++px) {
      uint32_t rng = sseed ^ (px * 1973u + py * 9277u * 65537u + 1013904223u);
      float acc = 0.0f;
      for (uint32_t sy = 0; sy < g; ++sy)
        for (uint32_t sx = 0; sx < g; ++sx) {
          const float sub_x = (static_cast<float>(sx) + rand_f32(rng)) / static_cast<float>(g);
          const float sub_y = (static_cast<float>(sy) + rand_f32(rng)) / static_cast<float>(g);
          const float fx = (static_cast<float>(px) + sub_x) * pw;
          const float fy = (static_cast<float>(py) + sub_y) * ph;
          const float orig[3] = {fx, fy, film_d + 0.1f};
          const float dir[3] = {0.0f, 0.0f, -1.0f};
          float total = 0.0f;
          const int cx = static_cast<int>(std::floor(fx / cs)), cy = static_cast<int>(std::floor(fy / cs));
          for (int dy = -2; dy <= 2; ++dy) {
            const int gy = cy + dy;
            if (gy < 0 || gy >= static_cast<int>(gh)) continue;
            for (int dx = -2; dx <= 2; ++dx) {
              const int gx = cx + dx;
              if (gx < 0 || gx >= static_cast<int>(gw)) continue;
              for (int gz = 0; gz < static_cast<int>(gd); ++gz) {
                const Cell& c = cells[(static_cast<size_t>(gz) * gh + gy) * gw + gx];
                if (c.flags[0] == 0u || c.flags[2] == 0u) continue;
                const float rel[3] = {orig[0] - c.pos[0], orig[1] - c.pos[1], orig[2] - c.pos[2]};
                float lo[3], ld[3];
                quat_inv_rot(c.rot, rel, lo);
                quat_inv_rot(c.rot, dir, ld);
                const float dims[3] = {c.dims_exp[0] * c.dims_exp[3], c.dims_exp[1] * c.dims_exp[3],
                                       c.dims_exp[2] * c.dims_exp[3]};
                if (c.flags[1] == 0u) {
                  float te = -INFINITY, tx = INFINITY;
                  float tmin[3], tmax[3];
                  for (int k = 0; k < 3; ++k) {
                    const float sgn = ld[k] > 0.0f ? 1.0f : (ld[k] < 0.0f ? -1.0f : 0.0f);
                    const float safe_sign = sgn == 0.0f ? 1.0f : sgn;
                    const float sd = std::fabs(ld[k]) < 1e-6f ? safe_sign * 1e-6f : ld[k];
                    const float inv = 1.0f / sd;
                    const float t1 = (-dims[k] - lo[k]) * inv, t2 = (dims[k] - lo[k]) * inv;
                    tmin[k] = std::fmin(t1, t2);
                    tmax[k] = std::fmax(t1, t2);
                  }
                  te = std::fmax(std::fmax(tmin[0], tmin[1]), tmin[2]);
                  tx = std::fmin(std::fmin(tmax[0], tmax[1]), tmax[2]);
                  if (tx >= te && tx > 0.0f) {
                    const float path = tx - std::fmax(te, 0.0f);
                    if (path > 0.0f) total += path;
                  }
                } else {
                  const float pp[3] = {lo[0] / dims[0], lo[1] / dims[1], lo[2] / dims[2]};
                  const float dd[3] = {ld[0] / dims[0], ld[1] / dims[1], ld[2] / dims[2]};
                  const float a = dot3(dd, dd);
                  if (a > 1e-6f) {
                    const float b = 2.0f * dot3(pp, dd);
                    const float cc = dot3(pp, pp) - 1.0f;
                    const float disc = b * b - 4.0f * a * cc;
                    if (disc >= 0.0f) {
                      const float sq = std::sqrt(disc);
                      const float inv2a = 0.5f / a;
                      const float t0 = (-b - sq) * inv2a, t1 = (-b + sq) * inv2a;
                      const float te = std::fmin(t0, t1), tx = std::fmax(t0, t1);
                      if (tx > 0.0f && tx >= te) {
                        const float path = tx - std::fmax(te, 0.0f);
                        if (path > 0.0f) total += path;
                      }
                    }
                  }
                }
              }
            }
          }
          const float safe = clampf(total, 0.0f, film_d);
          acc += fexp(-opacity * safe);
        }
      const float mean_t = clampf(acc / static_cast<float>(g * g), 1e-4f, 1.0f);
      d_neg[static_cast<size_t>(py) * W + px] = -flog(mean_t) / 2.302585092994046f + 0.05f;
    }
  if (cells_out) std::memcpy(cells_out, cells.data(), nc * sizeof(Cell));
  return 0;
}

}  // extern "C"
