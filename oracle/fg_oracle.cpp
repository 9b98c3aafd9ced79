// CPU oracle for the fgrain photon-transport and transmittance-scan path.
//
// TEST INFRASTRUCTURE ONLY: tests/ use this library as the checker for the CUDA library, and
// bench.py times it as the CPU baseline.  The product never links or calls it.
//
// Every stage restates the reference's Rust CPU code (paths relative to the fgrain project):
//   poisson.rs:14-132          Bridson 3D Poisson-disk sampling          -> sample_poisson
//   emulsion.rs:46-220         presets and crystal synthesis             -> synthesize
//   crystal.rs:106-223         AABB, ray/crystal intersection            -> crystal_aabb, intersect
//   bvh.rs:96-402              spatial-median BVH, any-hit walk, radius  -> RefBvh
//   optics.rs:75-196           gelatin optics                            -> free_path, hg, ...
//   transport.rs:48-188        Monte-Carlo exposure                      -> expose
//   development.rs:59-188      threshold + BFS clumping                  -> develop
//   transmittance.rs:65-171    scanner                                   -> scan
//   image_pipeline.rs:924-1014 tile worker                               -> or_render_tile
//   image_pipeline.rs:315-330, 593-649, 825-855 resize, Hann blend, OTF
// Floating point follows the reference: IEEE double, no contraction (built with
// -ffp-contract=off), NaN-ignoring min/max like Rust's f64::min/max (fmin/fmax).
// The only deliberate departure is the random stream (Philox-4x32-10, see philox.h).
#include "fg_oracle.h"

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <vector>

#include "philox.h"

namespace fgo {

struct V3 {
  double x, y, z;
};
static inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
// nalgebra's 3-vector dot sums the three products left to right.
static inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline V3 normalize(V3 a) {
  const double n = std::sqrt(dot(a, a));
  return v3(a.x / n, a.y / n, a.z / n);
}
static inline double rmin(double a, double b) { return std::fmin(a, b); }
static inline double rmax(double a, double b) { return std::fmax(a, b); }
static inline double rclamp(double v, double lo, double hi) { return rmin(rmax(v, lo), hi); }

// UnitQuaternion::inverse_transform_vector: rotate by the conjugate quaternion,
// v' = v + w t + q x t with t = 2 (q x v) and q the conjugated vector part.
static inline V3 quat_inv_rotate(const double* q, V3 v) {
  const V3 qv = v3(-q[0], -q[1], -q[2]);
  const double w = q[3];
  const V3 t = cross(qv, v) * 2.0;
  const V3 c = cross(qv, t);
  return (t * w + c) + v;
}

struct Crystal {
  V3 pos, dims;
  double q[4];
  int morph;
  double sens;
  bool developed;
  double fe;
};

static inline Crystal load_crystal(const or_crystals* c, size_t i) {
  Crystal k;
  k.pos = v3(c->pos[3 * i], c->pos[3 * i + 1], c->pos[3 * i + 2]);
  k.dims = v3(c->dims[3 * i], c->dims[3 * i + 1], c->dims[3 * i + 2]);
  for (int j = 0; j < 4; ++j) k.q[j] = c->quat[4 * i + j];
  k.morph = c->morph ? c->morph[i] : 0;
  k.sens = c->sens ? c->sens[i] : 1.0;
  k.developed = c->developed ? c->developed[i] != 0 : false;
  k.fe = c->expansion ? c->expansion[i] : 1.0;
  return k;
}

struct Box {
  V3 lo, hi;
};

// HalideCrystal::aabb (crystal.rs:106-133): a cube of half-side max_dim * expansion.
static inline Box crystal_aabb(const Crystal& k) {
  const double e = k.developed ? k.fe : 1.0;
  const double m = rmax(rmax(k.dims.x, k.dims.y), k.dims.z) * e;
  return Box{v3(k.pos.x - m, k.pos.y - m, k.pos.z - m), v3(k.pos.x + m, k.pos.y + m, k.pos.z + m)};
}

// AABB::intersect_ray (bvh.rs:96-124), Kay-Kajiya slabs with NaN-ignoring min/max.
static inline bool box_hit(const Box& b, V3 o, V3 inv) {
  const double t1x = (b.lo.x - o.x) * inv.x, t2x = (b.hi.x - o.x) * inv.x;
  const double t1y = (b.lo.y - o.y) * inv.y, t2y = (b.hi.y - o.y) * inv.y;
  const double t1z = (b.lo.z - o.z) * inv.z, t2z = (b.hi.z - o.z) * inv.z;
  const double te = rmax(rmax(rmin(t1x, t2x), rmin(t1y, t2y)), rmin(t1z, t2z));
  const double tx = rmin(rmin(rmax(t1x, t2x), rmax(t1y, t2y)), rmax(t1z, t2z));
  return tx >= te && tx > 0.0;
}

// HalideCrystal::intersect_ray (crystal.rs:140-217).
static inline bool intersect(const Crystal& k, V3 o, V3 d, double& t0, double& t1) {
  const double e = k.developed ? k.fe : 1.0;
  const V3 lo = quat_inv_rotate(k.q, o - k.pos);
  const V3 ld = quat_inv_rotate(k.q, d);
  const V3 dm = k.dims * e;
  if (k.morph == 0) {
    const V3 inv = v3(1.0 / ld.x, 1.0 / ld.y, 1.0 / ld.z);
    const double a1 = (-dm.x - lo.x) * inv.x, a2 = (dm.x - lo.x) * inv.x;
    const double b1 = (-dm.y - lo.y) * inv.y, b2 = (dm.y - lo.y) * inv.y;
    const double c1 = (-dm.z - lo.z) * inv.z, c2 = (dm.z - lo.z) * inv.z;
    const double tmin = rmax(rmax(rmin(a1, a2), rmin(b1, b2)), rmin(c1, c2));
    const double tmax = rmin(rmin(rmax(a1, a2), rmax(b1, b2)), rmax(c1, c2));
    if (tmax >= tmin && tmax > 0.0) {
      t0 = rmax(tmin, 0.0);
      t1 = tmax;
      return true;
    }
    return false;
  }
  const V3 p = v3(lo.x / dm.x, lo.y / dm.y, lo.z / dm.z);
  const V3 dd = v3(ld.x / dm.x, ld.y / dm.y, ld.z / dm.z);
  const double a = dot(dd, dd);
  const double b = 2.0 * dot(p, dd);
  const double c = dot(p, p) - 1.0;
  const double disc = b * b - 4.0 * a * c;
  if (disc < 0.0) return false;
  const double sq = std::sqrt(disc);
  const double r0 = (-b - sq) / (2.0 * a);
  const double r1 = (-b + sq) / (2.0 * a);
  const double te = rmin(r0, r1), tx = rmax(r0, r1);
  if (tx > 0.0) {
    t0 = rmax(te, 0.0);
    t1 = tx;
    return true;
  }
  return false;
}

// ---------------------------------------------------------------------------------------------
// Reference BVH (bvh.rs:129-402): top-down spatial median, leaves of at most four crystals,
// 64-entry traversal stack that silently drops children on overflow.
struct Node {
  Box box;
  uint32_t left, right, offset, count;
};

struct RefBvh {
  std::vector<Node> nodes;
  std::vector<size_t> indices;
  int64_t depth = 0;

  static Box unite(const Box& a, const Box& b) {
    return Box{v3(rmin(a.lo.x, b.lo.x), rmin(a.lo.y, b.lo.y), rmin(a.lo.z, b.lo.z)),
               v3(rmax(a.hi.x, b.hi.x), rmax(a.hi.y, b.hi.y), rmax(a.hi.z, b.hi.z))};
  }

  void build(const std::vector<Crystal>& cs) {
    nodes.clear();
    indices.clear();
    if (cs.empty()) return;
    indices.resize(cs.size());
    for (size_t i = 0; i < cs.size(); ++i) indices[i] = i;
    nodes.reserve(cs.size() * 2);
    std::vector<Box> boxes(cs.size());
    std::vector<V3> cent(cs.size());
    for (size_t i = 0; i < cs.size(); ++i) {
      boxes[i] = crystal_aabb(cs[i]);
      cent[i] = v3(0.5 * (boxes[i].lo.x + boxes[i].hi.x), 0.5 * (boxes[i].lo.y + boxes[i].hi.y),
                   0.5 * (boxes[i].lo.z + boxes[i].hi.z));
    }
    subdivide(boxes, cent, 0, cs.size(), 1);
  }

  uint32_t subdivide(const std::vector<Box>& boxes, const std::vector<V3>& cent, size_t start,
                     size_t count, int64_t level) {
    depth = std::max(depth, level);
    const uint32_t idx = static_cast<uint32_t>(nodes.size());
    const double inf = INFINITY;
    Box all{v3(inf, inf, inf), v3(-inf, -inf, -inf)};
    Box cb = all;
    for (size_t k = start; k < start + count; ++k) {
      const size_t i = indices[k];
      all = unite(all, boxes[i]);
      cb = unite(cb, Box{cent[i], cent[i]});
    }
    if (count <= 4) {
      nodes.push_back(Node{all, 0, 0, static_cast<uint32_t>(start), static_cast<uint32_t>(count)});
      return idx;
    }
    const V3 ext = cb.hi - cb.lo;
    int axis;
    if (ext.x >= ext.y && ext.x >= ext.z)
      axis = 0;
    else if (ext.y >= ext.z)
      axis = 1;
    else
      axis = 2;
    auto comp = [axis](const V3& v) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); };
    if (comp(ext) <= 1e-7) {
      nodes.push_back(Node{all, 0, 0, static_cast<uint32_t>(start), static_cast<uint32_t>(count)});
      return idx;
    }
    // Two-pointer partition around the centroid-box midpoint (bvh.rs:210-225): elements below
    // the midpoint stay in front; others are swapped to the back.
    const double mid = 0.5 * (comp(cb.lo) + comp(cb.hi));
    size_t i = start, j = start + count - 1;
    while (i <= j) {
      if (comp(cent[indices[i]]) < mid) {
        ++i;
      } else {
        std::swap(indices[i], indices[j]);
        if (j == 0) break;
        --j;
      }
    }
    const size_t left_count = i - start;
    const size_t split = (left_count == 0 || left_count == count) ? count / 2 : left_count;
    nodes.push_back(Node{all, 0, 0, 0, 0});
    const uint32_t l = subdivide(boxes, cent, start, split, level + 1);
    const uint32_t r = subdivide(boxes, cent, start + split, count - split, level + 1);
    nodes[idx].left = l;
    nodes[idx].right = r;
    return idx;
  }

  // BVH::intersect_ray_all (bvh.rs:300-347).  fn(leaf_index) is called for each leaf hit in
  // traversal order; returns the number of dropped pushes.
  template <class F>
  int64_t walk(V3 o, V3 d, F&& fn) const {
    if (nodes.empty()) return 0;
    const V3 inv = v3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    int64_t dropped = 0;
    while (sp > 0) {
      const Node& n = nodes[stack[--sp]];
      if (!box_hit(n.box, o, inv)) continue;
      if (n.count > 0) {
        for (uint32_t k = n.offset; k < n.offset + n.count; ++k) fn(indices[k]);
      } else if (sp + 2 < 64) {
        stack[sp] = n.left;
        stack[sp + 1] = n.right;
        sp += 2;
      } else {
        ++dropped;
      }
    }
    return dropped;
  }

  // BVH::query_radius (bvh.rs:350-402).
  void query_radius(const std::vector<Crystal>& cs, V3 c, double r,
                    std::vector<size_t>& out) const {
    if (nodes.empty()) return;
    const double r2 = r * r;
    const Box q{v3(c.x - r, c.y - r, c.z - r), v3(c.x + r, c.y + r, c.z + r)};
    uint32_t stack[64];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
      const Node& n = nodes[stack[--sp]];
      const bool ov = n.box.lo.x <= q.hi.x && n.box.hi.x >= q.lo.x && n.box.lo.y <= q.hi.y &&
                      n.box.hi.y >= q.lo.y && n.box.lo.z <= q.hi.z && n.box.hi.z >= q.lo.z;
      if (!ov) continue;
      if (n.count > 0) {
        for (uint32_t k = n.offset; k < n.offset + n.count; ++k) {
          const size_t ci = indices[k];
          const V3 df = cs[ci].pos - c;
          if (dot(df, df) <= r2) out.push_back(ci);
        }
      } else if (sp + 2 < 64) {
        stack[sp] = n.left;
        stack[sp + 1] = n.right;
        sp += 2;
      }
    }
  }
};

struct Hit {
  size_t idx;
  double t0, t1;
};

// All hits of one ray under the chosen rule.  CANONICAL sorts by (t_enter, index).
static void ray_hits(const RefBvh& bvh, const std::vector<Crystal>& cs, V3 o, V3 d, int mode,
                     std::vector<Hit>& out) {
  out.clear();
  const V3 inv = v3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
  bvh.walk(o, d, [&](size_t i) {
    double t0, t1;
    if (!intersect(cs[i], o, d, t0, t1)) return;
    if (mode == OR_CANONICAL && !box_hit(crystal_aabb(cs[i]), o, inv)) return;
    out.push_back(Hit{i, t0, t1});
  });
  if (mode == OR_CANONICAL) {
    std::sort(out.begin(), out.end(), [](const Hit& a, const Hit& b) {
      return a.t0 < b.t0 || (a.t0 == b.t0 && a.idx < b.idx);
    });
  }
}

static std::vector<Crystal> load_all(const or_crystals* c) {
  std::vector<Crystal> cs(c->n);
  for (size_t i = 0; i < c->n; ++i) cs[i] = load_crystal(c, i);
  return cs;
}

// ---------------------------------------------------------------------------------------------
// Gelatin optics (optics.rs:75-196).
struct Optics {
  or_optics o;
  double mu_t() const { return o.absorption_coeff + o.scattering_coeff; }
  double albedo() const {
    const double mt = mu_t();
    return mt > 0.0 ? o.scattering_coeff / mt : 0.0;
  }
  double free_path(double xi) const {
    const double mt = mu_t();
    if (mt <= 0.0) return 1e6;
    return -std::log(rmax(1.0 - xi, 2.2250738585072014e-308)) / mt;
  }
  V3 hg(V3 cur, double xi1, double xi2) const {
    const double g = o.anisotropy_g;
    double ct;
    if (std::fabs(g) < 1e-4) {
      ct = 2.0 * xi1 - 1.0;
    } else {
      const double term = (1.0 - g * g) / (1.0 - g + 2.0 * g * xi1);
      ct = (1.0 + g * g - term * term) / (2.0 * g);
    }
    ct = rclamp(ct, -1.0, 1.0);
    const double st = std::sqrt(rmax(1.0 - ct * ct, 0.0));
    const double phi = 2.0 * M_PI * xi2;
    const V3 w = normalize(cur);
    const V3 u = std::fabs(w.x) > 0.1 ? normalize(cross(v3(0, 1, 0), w))
                                      : normalize(cross(v3(1, 0, 0), w));
    const V3 vv = cross(w, u);
    return normalize((u * (st * std::cos(phi)) + vv * (st * std::sin(phi))) + w * ct);
  }
  double fresnel(double cos_i) const {
    const double n1 = 1.0, n2 = o.refractive_index;
    const double r = (n1 - n2) / (n1 + n2);
    const double r0 = r * r;
    const double c = rclamp(std::fabs(cos_i), 0.0, 1.0);
    const double m = 1.0 - c;
    const double m2 = m * m;
    return r0 + (1.0 - r0) * (m2 * m2 * m);
  }
};

// ---------------------------------------------------------------------------------------------
// Bridson sampling (poisson.rs:14-132) on a sequential Philox stream.
static std::vector<V3> sample_poisson(V3 b, double r_min, uint32_t k, PhiloxStream& rng) {
  std::vector<V3> pts;
  if (b.x <= 0.0 || b.y <= 0.0 || b.z <= 0.0 || r_min <= 0.0) return pts;
  const double cell = r_min / std::sqrt(3.0);
  const int64_t gw = static_cast<int64_t>(std::ceil(b.x / cell));
  const int64_t gh = static_cast<int64_t>(std::ceil(b.y / cell));
  const int64_t gd = static_cast<int64_t>(std::ceil(b.z / cell));
  std::vector<int64_t> grid(static_cast<size_t>(gw * gh * gd), -1);
  auto gidx = [&](int64_t x, int64_t y, int64_t z) { return x + y * gw + z * gw * gh; };
  auto to_grid = [&](V3 p, int64_t& x, int64_t& y, int64_t& z) {
    x = std::clamp(static_cast<int64_t>(std::floor(p.x / cell)), int64_t(0), gw - 1);
    y = std::clamp(static_cast<int64_t>(std::floor(p.y / cell)), int64_t(0), gh - 1);
    z = std::clamp(static_cast<int64_t>(std::floor(p.z / cell)), int64_t(0), gd - 1);
  };
  std::vector<size_t> active;
  const double fx = rng.uniform() * b.x;
  const double fy = rng.uniform() * b.y;
  const double fz = rng.uniform() * b.z;
  const V3 first = v3(fx, fy, fz);
  int64_t gx, gy, gz;
  to_grid(first, gx, gy, gz);
  grid[gidx(gx, gy, gz)] = 0;
  pts.push_back(first);
  active.push_back(0);
  const double r2 = r_min * r_min;
  while (!active.empty()) {
    const size_t pick = static_cast<size_t>(rng.below(active.size()));
    const V3 base = pts[active[pick]];
    bool found = false;
    for (uint32_t s = 0; s < k; ++s) {
      const double u = rng.uniform();
      const double ct = rng.uniform() * 2.0 + -1.0;
      const double st = std::sqrt(rmax(1.0 - ct * ct, 0.0));
      const double phi = rng.uniform() * (2.0 * M_PI);
      const double rad = std::cbrt(7.0 * u + 1.0) * r_min;
      const V3 c = v3(base.x + rad * st * std::cos(phi), base.y + rad * st * std::sin(phi),
                      base.z + rad * ct);
      if (c.x < 0.0 || c.x >= b.x || c.y < 0.0 || c.y >= b.y || c.z < 0.0 || c.z >= b.z) continue;
      int64_t cx, cy, cz;
      to_grid(c, cx, cy, cz);
      bool close = false;
      for (int64_t z = std::max<int64_t>(cz - 2, 0); z <= std::min(cz + 2, gd - 1) && !close; ++z)
        for (int64_t y = std::max<int64_t>(cy - 2, 0); y <= std::min(cy + 2, gh - 1) && !close; ++y)
          for (int64_t x = std::max<int64_t>(cx - 2, 0); x <= std::min(cx + 2, gw - 1); ++x) {
            const int64_t e = grid[gidx(x, y, z)];
            if (e >= 0) {
              const V3 df = pts[e] - c;
              if (dot(df, df) < r2) {
                close = true;
                break;
              }
            }
          }
      if (!close) {
        grid[gidx(cx, cy, cz)] = static_cast<int64_t>(pts.size());
        active.push_back(pts.size());
        pts.push_back(c);
        found = true;
        break;
      }
    }
    if (!found) {
      active[pick] = active.back();
      active.pop_back();
    }
  }
  return pts;
}

// Standard normal from two uniforms (Box-Muller, cosine branch).  The reference draws its
// normals with rand_distr's ziggurat; only the distribution is shared.
static inline double std_normal(PhiloxStream& rng) {
  const double u1 = 1.0 - rng.uniform();
  const double u2 = rng.uniform();
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

}  // namespace fgo

using namespace fgo;

// =============================================================================================
extern "C" {

int or_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
              uint32_t out[4]) {
  const Philox4 r = philox4x32_10(c0, c1, c2, c3, k0, k1);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
  return 0;
}

int or_intersect_crystal(const double pos[3], const double dims[3], const double quat[4],
                         int32_t morph, double expansion, const double origin[3],
                         const double dir[3], double* t_enter, double* t_exit) {
  Crystal k;
  k.pos = v3(pos[0], pos[1], pos[2]);
  k.dims = v3(dims[0], dims[1], dims[2]);
  for (int j = 0; j < 4; ++j) k.q[j] = quat[j];
  k.morph = morph;
  k.sens = 1.0;
  k.developed = expansion != 1.0;
  k.fe = expansion;
  double t0 = 0, t1 = 0;
  const bool h = intersect(k, v3(origin[0], origin[1], origin[2]), v3(dir[0], dir[1], dir[2]), t0, t1);
  if (h) {
    *t_enter = t0;
    *t_exit = t1;
  }
  return h ? 1 : 0;
}

int64_t or_ray_hits(const or_crystals* c, const double origin[3], const double dir[3], int mode,
                    uint32_t* idx_out, double* t0_out, double* t1_out, int64_t cap) {
  const std::vector<Crystal> cs = load_all(c);
  RefBvh bvh;
  bvh.build(cs);
  std::vector<Hit> hits;
  ray_hits(bvh, cs, v3(origin[0], origin[1], origin[2]), v3(dir[0], dir[1], dir[2]), mode, hits);
  for (int64_t i = 0; i < static_cast<int64_t>(hits.size()) && i < cap; ++i) {
    idx_out[i] = static_cast<uint32_t>(hits[i].idx);
    if (t0_out) t0_out[i] = hits[i].t0;
    if (t1_out) t1_out[i] = hits[i].t1;
  }
  return static_cast<int64_t>(hits.size());
}

int64_t or_query_radius(const or_crystals* c, const double center[3], double radius,
                        uint32_t* out, int64_t cap) {
  const std::vector<Crystal> cs = load_all(c);
  RefBvh bvh;
  bvh.build(cs);
  std::vector<size_t> res;
  bvh.query_radius(cs, v3(center[0], center[1], center[2]), radius, res);
  for (int64_t i = 0; i < static_cast<int64_t>(res.size()) && i < cap; ++i)
    out[i] = static_cast<uint32_t>(res[i]);
  return static_cast<int64_t>(res.size());
}

int or_bvh_stats(const or_crystals* c, int64_t* nodes, int64_t* depth) {
  const std::vector<Crystal> cs = load_all(c);
  RefBvh bvh;
  bvh.build(cs);
  *nodes = static_cast<int64_t>(bvh.nodes.size());
  *depth = bvh.depth;
  return 0;
}

// The reference tree over all crystals, or over the developed ones only (the scan's tree,
// transmittance.rs:86-89): the final index order (crystal indices), and per leaf in node order its
// range in that order and its box.  Returns the number of elements.
int64_t or_bvh_export(const or_crystals* c, int developed_only, uint32_t* order, int64_t cap,
                      uint32_t* leaf_start, uint32_t* leaf_count, double* leaf_box, int64_t leaf_cap,
                      int64_t* nleaves) {
  std::vector<Crystal> cs;
  std::vector<size_t> orig;
  for (size_t i = 0; i < c->n; ++i) {
    Crystal k = load_crystal(c, i);
    if (developed_only && !k.developed) continue;
    if (!developed_only) k.developed = false;
    cs.push_back(k);
    orig.push_back(i);
  }
  RefBvh bvh;
  bvh.build(cs);
  for (size_t k = 0; k < bvh.indices.size() && static_cast<int64_t>(k) < cap; ++k)
    order[k] = static_cast<uint32_t>(orig[bvh.indices[k]]);
  int64_t nl = 0;
  for (const auto& n : bvh.nodes) {
    if (n.count == 0) continue;
    if (nl < leaf_cap) {
      leaf_start[nl] = n.offset;
      leaf_count[nl] = n.count;
      const double b[6] = {n.box.lo.x, n.box.lo.y, n.box.lo.z, n.box.hi.x, n.box.hi.y, n.box.hi.z};
      for (int j = 0; j < 6; ++j) leaf_box[6 * nl + j] = b[j];
    }
    ++nl;
  }
  *nleaves = nl;
  return static_cast<int64_t>(cs.size());
}

double or_free_path(const or_optics* o, double xi) { return Optics{*o}.free_path(xi); }

int or_antihalation(const or_optics* o, double* energy, double dir[3], const double u[4]) {
  const double dye_t = std::pow(10.0, -2.0 * o->antihalation_density);
  double E = *energy * (o->antihalation_reflectance * dye_t);
  V3 d = v3(dir[0], dir[1], dir[2]);
  if (E < 1e-4) {
    if (u[0] < 0.1) {
      E /= 0.1;
    } else {
      *energy = E;
      return 0;
    }
  }
  if (u[1] < 0.4) {
    const double r = std::sqrt(u[2]);
    const double ph = 2.0 * M_PI * u[3];
    d = normalize(v3(r * std::cos(ph), r * std::sin(ph), -std::sqrt(rmax(1.0 - u[2], 0.0))));
  } else {
    d.z = -std::fabs(d.z);
    d = normalize(d);
  }
  *energy = E;
  dir[0] = d.x;
  dir[1] = d.y;
  dir[2] = d.z;
  return 1;
}

int64_t or_rays_hits(const or_crystals* c, const double* origins, const double* dirs, int64_t n,
                     int mode, int developed_only, uint32_t* offsets, uint32_t* ids,
                     int64_t id_cap, double* chord_sum) {
  std::vector<Crystal> all = load_all(c), sub;
  std::vector<size_t> orig;
  for (size_t i = 0; i < all.size(); ++i) {
    if (developed_only && !all[i].developed) continue;
    if (!developed_only) all[i].developed = false;
    sub.push_back(all[i]);
    orig.push_back(i);
  }
  RefBvh bvh;
  bvh.build(sub);
  std::vector<std::vector<uint32_t>> lists(static_cast<size_t>(n));
  std::vector<double> L(static_cast<size_t>(n), 0.0);
#pragma omp parallel
  {
    std::vector<Hit> hits;
#pragma omp for schedule(dynamic, 64)
    for (int64_t r = 0; r < n; ++r) {
      if (sub.empty()) continue;
      ray_hits(bvh, sub, v3(origins[3 * r], origins[3 * r + 1], origins[3 * r + 2]),
               v3(dirs[3 * r], dirs[3 * r + 1], dirs[3 * r + 2]), mode, hits);
      double acc = 0.0;
      for (const Hit& h : hits) {
        lists[r].push_back(static_cast<uint32_t>(orig[h.idx]));
        acc += rmax(h.t1 - h.t0, 0.0);
      }
      L[r] = acc;
    }
  }
  int64_t total = 0;
  for (int64_t r = 0; r < n; ++r) {
    if (offsets) offsets[r] = static_cast<uint32_t>(total);
    for (uint32_t id : lists[r]) {
      if (ids && total < id_cap) ids[total] = id;
      ++total;
    }
    if (chord_sum) chord_sum[r] = L[r];
  }
  if (offsets) offsets[n] = static_cast<uint32_t>(total);
  return total;
}

int64_t or_sample_poisson(const double bounds[3], double r_min, uint32_t k, uint64_t seed,
                          double* pts, int64_t cap) {
  PhiloxStream rng(seed, TAG_SYNTH);
  const std::vector<V3> p = sample_poisson(v3(bounds[0], bounds[1], bounds[2]), r_min, k, rng);
  for (int64_t i = 0; i < static_cast<int64_t>(p.size()) && i < cap; ++i) {
    pts[3 * i] = p[i].x;
    pts[3 * i + 1] = p[i].y;
    pts[3 * i + 2] = p[i].z;
  }
  return static_cast<int64_t>(p.size());
}

int64_t or_synthesize(const or_emulsion_cfg* cfg, uint64_t seed, or_crystals* out) {
  PhiloxStream rng(seed, TAG_SYNTH);
  const std::vector<V3> pts =
      sample_poisson(v3(cfg->width, cfg->height, cfg->depth), cfg->r_min, 30, rng);
  const int64_t n = static_cast<int64_t>(pts.size());
  if (n > static_cast<int64_t>(out->n)) return n;  // caller retries with enough room
  // LogNormal::new(ln mean, sigma) falls back to (0, 0.2) when the parameters are invalid.
  double mu = std::log(cfg->mean_crystal_radius), sg = cfg->size_variance;
  if (!(sg >= 0.0) || !std::isfinite(mu) || !std::isfinite(sg)) {
    mu = 0.0;
    sg = 0.2;
  }
  for (int64_t i = 0; i < n; ++i) {
    const double radius = rclamp(std::exp(mu + sg * std_normal(rng)), 0.15, cfg->r_min * 0.48);
    const double sens = rmax(cfg->base_sensitivity + 0.15 * std_normal(rng), 0.1);
    double q[4];
    V3 dims;
    if (cfg->morphology == 0 || cfg->morphology == 2) {
      const double u1 = rng.uniform(), u2 = rng.uniform(), u3 = rng.uniform();
      const double roll = u1 * (2.0 * M_PI), pitch = u2 * M_PI, yaw = u3 * (2.0 * M_PI);
      const double sr = std::sin(roll * 0.5), cr = std::cos(roll * 0.5);
      const double sp = std::sin(pitch * 0.5), cp = std::cos(pitch * 0.5);
      const double sy = std::sin(yaw * 0.5), cy = std::cos(yaw * 0.5);
      q[3] = cr * cp * cy + sr * sp * sy;
      q[0] = sr * cp * cy - cr * sp * sy;
      q[1] = cr * sp * cy + sr * cp * sy;
      q[2] = cr * cp * sy - sr * sp * cy;
      dims = v3(radius, radius, radius);
    } else {
      const double ht = rmax(radius / cfg->tabular_aspect_ratio, 0.05);
      const double tilt = rng.uniform() * 0.34 + -0.17;
      const double ax = rng.uniform() * 2.0 + -1.0;
      const double ay = rng.uniform() * 2.0 + -1.0;
      const V3 axis = normalize(normalize(v3(ax, ay, 0.0)));
      const double s = std::sin(tilt / 2.0), c = std::cos(tilt / 2.0);
      q[0] = axis.x * s;
      q[1] = axis.y * s;
      q[2] = axis.z * s;
      q[3] = c;
      dims = v3(radius, radius, ht);
    }
    out->pos[3 * i] = pts[i].x;
    out->pos[3 * i + 1] = pts[i].y;
    out->pos[3 * i + 2] = pts[i].z;
    out->dims[3 * i] = dims.x;
    out->dims[3 * i + 1] = dims.y;
    out->dims[3 * i + 2] = dims.z;
    for (int j = 0; j < 4; ++j) out->quat[4 * i + j] = q[j];
    out->sens[i] = sens;
    out->morph[i] = cfg->morphology;
    if (out->latent) out->latent[i] = 0;
    if (out->developed) out->developed[i] = 0;
    if (out->clump) out->clump[i] = -1;
    if (out->expansion) out->expansion[i] = 1.0;
  }
  out->n = static_cast<size_t>(n);
  return n;
}

// Per-hit Beer-Lambert absorption and Bernoulli rounding (transport.rs:108-138).  Returns the
// new energy; *count receives the latent photons to record.
static inline double absorb(double energy, double path, double alpha, double sens, double u,
                            uint32_t* count) {
  const double p_abs = 1.0 - std::exp(-alpha * path);
  const double absorbed = energy * p_abs * sens;
  const double expected = absorbed * 5.0;
  const double fl = std::floor(expected);
  const uint32_t whole = fl <= 0.0 ? 0u : (fl >= 4294967295.0 ? 4294967295u : static_cast<uint32_t>(fl));
  const double frac = expected - static_cast<double>(whole);
  const uint32_t extra = (u < rclamp(frac, 0.0, 1.0)) ? 1u : 0u;
  *count = whole + extra;
  return energy * rmax(1.0 - p_abs * 0.9, 0.05);
}

static inline double hit_uniform(uint32_t k0, uint32_t k1, uint32_t pid, uint32_t bounce,
                                 uint32_t ordinal) {
  const Philox4 r = philox4x32_10(pid, bounce, ordinal >> 2, TAG_HIT, k0, k1);
  return u24(r.v[ordinal & 3]);
}

int64_t or_expose(or_crystals* c, const or_emulsion_cfg* cfg, const float* tile, uint32_t tw,
                  uint32_t th, const or_exposure_cfg* ecfg, uint64_t seed, int mode,
                  int threads, or_segment* seg_out, int64_t seg_cap, int64_t* seg_n,
                  uint64_t* hits_out) {
  const std::vector<Crystal> cs = load_all(c);
  RefBvh bvh;
  bvh.build(cs);
  const double W = cfg->width, H = cfg->height, D = cfg->depth;
  const double area = W * H;
  const int64_t P = static_cast<int64_t>(std::round(area * ecfg->photons_per_sq_um));
  if (seg_n) *seg_n = 0;
  if (hits_out) *hits_out = 0;
  if (P <= 0) return 0;
  const Optics opt{cfg->optics};
  const uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
  const double dye_t = std::pow(10.0, -2.0 * opt.o.antihalation_density);
  const double eff_r = opt.o.antihalation_reflectance * dye_t;
  const double albedo = opt.albedo();
  std::vector<std::atomic<uint32_t>> lat(cs.size());
  for (size_t i = 0; i < cs.size(); ++i) lat[i].store(c->latent ? c->latent[i] : 0u);
  const int nt = threads > 0 ? threads : omp_get_max_threads();
  std::vector<std::vector<or_segment>> segs(static_cast<size_t>(nt));
  std::atomic<uint64_t> total_hits{0};

#pragma omp parallel num_threads(nt)
  {
    const int tid = omp_get_thread_num();
    std::vector<Hit> hits;
    uint64_t my_hits = 0;
#pragma omp for schedule(dynamic, 256)
    for (int64_t pid = 0; pid < P; ++pid) {
      const uint32_t id = static_cast<uint32_t>(pid);
      const Philox4 e0 = philox4x32_10(id, 0, 0, TAG_EMIT, k0, k1);
      const double x = u24(e0.v[0]) * W;
      const double y = u24(e0.v[1]) * H;
      // Nearest-pixel exposure closure of the tile worker (image_pipeline.rs:949-958).
      const double uu = rclamp(x / W, 0.0, 1.0), vv = rclamp(y / H, 0.0, 1.0);
      uint32_t px = static_cast<uint32_t>(std::round(uu * static_cast<double>(tw - 1)));
      uint32_t py = static_cast<uint32_t>(std::round(vv * static_cast<double>(th - 1)));
      px = std::min(px, tw - 1);
      py = std::min(py, th - 1);
      const double irr = rmax(static_cast<double>(tile[static_cast<size_t>(py) * tw + px]), 0.0);
      if (irr <= 0.0) continue;
      const double theta = u24(e0.v[2]) * ecfg->illumination_angle_rad;
      const double phi = u24(e0.v[3]) * (2.0 * M_PI);
      const double st = std::sin(theta);
      V3 dir = normalize(v3(st * std::cos(phi), st * std::sin(phi), std::cos(theta)));
      const Philox4 e1 = philox4x32_10(id, 0, 1, TAG_EMIT, k0, k1);
      if (u24(e1.v[0]) < opt.fresnel(dir.z)) continue;
      V3 pos = v3(x, y, 0.001);
      dir = normalize(dir);  // PhotonPacket::new normalises again
      double E = irr;
      bool alive = true;
      uint32_t b = 0;
      while (alive && b < ecfg->max_bounces) {
        const uint32_t bounce = b++;
        const Philox4 rb = philox4x32_10(id, bounce, 0, TAG_BOUNCE, k0, k1);
        const double step = rmin(opt.free_path(u24(rb.v[0])), D * 1.5);
        if (seg_out || seg_n) {
          or_segment s;
          s.origin[0] = pos.x; s.origin[1] = pos.y; s.origin[2] = pos.z;
          s.dir[0] = dir.x; s.dir[1] = dir.y; s.dir[2] = dir.z;
          s.step = step;
          s.energy = E;
          s.photon = id;
          s.bounce = bounce;
          segs[static_cast<size_t>(tid)].push_back(s);
        }
        ray_hits(bvh, cs, pos, dir, mode, hits);
        uint32_t ordinal = 0;
        for (const Hit& h : hits) {
          if (!(h.t0 < step)) continue;
          const double path = rmax(rmin(h.t1, step) - h.t0, 0.0);
          if (!(path > 0.0)) continue;
          uint32_t cnt;
          const double u = hit_uniform(k0, k1, id, bounce, ordinal++);
          E = absorb(E, path, ecfg->crystal_absorption_coeff, cs[h.idx].sens, u, &cnt);
          ++my_hits;
          if (cnt > 0) lat[h.idx].fetch_add(cnt, std::memory_order_relaxed);
        }
        const V3 np = pos + dir * step;
        if (np.x < 0.0 || np.x >= W || np.y < 0.0 || np.y >= H) break;
        if (np.z <= 0.0) break;
        if (np.z >= D) {
          pos = v3(np.x, np.y, D - 0.001);
          const Philox4 ra = philox4x32_10(id, bounce, 0, TAG_AH, k0, k1);
          E *= eff_r;
          if (E < 1e-4) {
            if (u24(ra.v[0]) < 0.1) {
              E /= 0.1;
            } else {
              alive = false;
              continue;
            }
          }
          if (u24(ra.v[1]) < 0.4) {
            const double u1 = u24(ra.v[2]), u2 = u24(ra.v[3]);
            const double r = std::sqrt(u1);
            const double ph = 2.0 * M_PI * u2;
            dir = normalize(v3(r * std::cos(ph), r * std::sin(ph), -std::sqrt(rmax(1.0 - u1, 0.0))));
          } else {
            dir.z = -std::fabs(dir.z);
            dir = normalize(dir);
          }
          continue;
        }
        pos = np;
        dir = opt.hg(dir, u24(rb.v[1]), u24(rb.v[2]));
        E *= albedo;
        if (E < 1e-3) {
          if (u24(rb.v[3]) < 0.1) {
            E /= 0.1;
          } else {
            break;
          }
        }
      }
    }
    total_hits.fetch_add(my_hits);
  }
  if (c->latent)
    for (size_t i = 0; i < cs.size(); ++i) c->latent[i] = lat[i].load();
  if (hits_out) *hits_out = total_hits.load();
  if (seg_out || seg_n) {
    std::vector<or_segment> all;
    for (auto& v : segs) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end(), [](const or_segment& a, const or_segment& b) {
      return a.photon < b.photon || (a.photon == b.photon && a.bounce < b.bounce);
    });
    if (seg_n) *seg_n = static_cast<int64_t>(all.size());
    if (seg_out)
      for (int64_t i = 0; i < static_cast<int64_t>(all.size()) && i < seg_cap; ++i) seg_out[i] = all[i];
  }
  return P;
}

int64_t or_replay_segments(or_crystals* c, const or_exposure_cfg* ecfg, uint64_t seed,
                           const or_segment* segs, int64_t nseg, int mode, uint32_t* offsets,
                           uint32_t* ids, int64_t id_cap) {
  const std::vector<Crystal> cs = load_all(c);
  RefBvh bvh;
  bvh.build(cs);
  const uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
  std::vector<Hit> hits;
  int64_t total = 0;
  for (int64_t s = 0; s < nseg; ++s) {
    const or_segment& g = segs[s];
    const V3 o = v3(g.origin[0], g.origin[1], g.origin[2]);
    const V3 d = v3(g.dir[0], g.dir[1], g.dir[2]);
    ray_hits(bvh, cs, o, d, mode, hits);
    if (offsets) offsets[s] = static_cast<uint32_t>(total);
    double E = g.energy;
    uint32_t ordinal = 0;
    for (const Hit& h : hits) {
      if (!(h.t0 < g.step)) continue;
      const double path = rmax(rmin(h.t1, g.step) - h.t0, 0.0);
      if (!(path > 0.0)) continue;
      uint32_t cnt;
      const double u = hit_uniform(k0, k1, g.photon, g.bounce, ordinal++);
      E = absorb(E, path, ecfg->crystal_absorption_coeff, cs[h.idx].sens, u, &cnt);
      if (c->latent && cnt > 0) c->latent[h.idx] += cnt;
      if (ids && total < id_cap) ids[total] = static_cast<uint32_t>(h.idx);
      ++total;
    }
  }
  if (offsets) offsets[nseg] = static_cast<uint32_t>(total);
  return total;
}

int or_develop(or_crystals* c, const or_dev_cfg* cfg, or_dev_report* rep) {
  std::memset(rep, 0, sizeof(*rep));
  const size_t n = c->n;
  if (n == 0) return 0;
  std::vector<Crystal> cs = load_all(c);
  // The BVH handed to develop_emulsion is the one built at synthesis (undeveloped boxes).
  for (auto& k : cs) {
    k.developed = false;
    k.fe = 1.0;
  }
  RefBvh bvh;
  bvh.build(cs);
  std::vector<double> fe(n);
  std::vector<uint8_t> dev(n);
  uint64_t developed = 0;
  for (size_t i = 0; i < n; ++i) {
    if (c->latent[i] >= cfg->threshold_photons) {
      dev[i] = 1;
      fe[i] = cfg->filament_expansion;
      ++developed;
    } else {
      dev[i] = 0;
      fe[i] = 0.0;
    }
    c->clump[i] = -1;
  }
  auto maxdim = [&](size_t i) { return rmax(rmax(cs[i].dims.x, cs[i].dims.y), cs[i].dims.z); };
  double max_base = 0.0;
  for (size_t i = 0; i < n; ++i) max_base = rmax(max_base, maxdim(i));
  std::vector<uint8_t> visited(n, 0);
  std::vector<size_t> queue, members, nb;
  uint64_t clumps = 0, max_size = 0, total_clumped = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!dev[i] || visited[i]) continue;
    const int64_t cid = static_cast<int64_t>(clumps++);
    visited[i] = 1;
    c->clump[i] = cid;
    queue.clear();
    size_t head = 0;
    queue.push_back(i);
    members.clear();
    members.push_back(i);
    while (head < queue.size()) {
      const size_t cur = queue[head++];
      const V3 cp = cs[cur].pos;
      const double rc = maxdim(cur) * fe[cur];
      const double search = (rc + max_base * cfg->filament_expansion) * cfg->clumping_proximity_factor;
      nb.clear();
      bvh.query_radius(cs, cp, search, nb);
      for (size_t j : nb) {
        if (j == cur || visited[j] || !dev[j]) continue;
        const double rn = maxdim(j) * fe[j];
        const double touch = (rc + rn) * cfg->clumping_proximity_factor;
        const V3 df = cs[j].pos - cp;
        if (dot(df, df) <= touch * touch) {
          visited[j] = 1;
          c->clump[j] = cid;
          queue.push_back(j);
          members.push_back(j);
        }
      }
    }
    const uint64_t sz = members.size();
    max_size = std::max(max_size, sz);
    total_clumped += sz;
    if (sz > 1) {
      const double boost = 1.15 + 0.18 * static_cast<double>(std::min<uint64_t>(sz, 6) - 1);
      for (size_t m : members) fe[m] *= boost;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    c->developed[i] = dev[i];
    c->expansion[i] = fe[i];
  }
  rep->total_crystals = n;
  rep->developed_crystals = developed;
  rep->fixed_crystals = n - developed;
  rep->total_clumps = clumps;
  rep->max_clump_size = max_size;
  rep->avg_clump_size = clumps > 0 ? static_cast<double>(total_clumped) / static_cast<double>(clumps) : 0.0;
  return 0;
}

static inline uint64_t pixel_seed(uint64_t seed, uint32_t px, uint32_t py) {
  return seed + static_cast<uint64_t>(px) * 0x9E3779B97F4A7C15ull +
         static_cast<uint64_t>(py) * 0xC6A4A7935BD1E995ull;
}

// Ray origin of stratum (sx, sy) of pixel (px, py) (transmittance.rs:102-120).
static inline V3 scan_origin(uint64_t seed, uint32_t px, uint32_t py, uint32_t sx, uint32_t sy,
                             uint32_t g, double pw, double ph, double z0) {
  const uint64_t ps = pixel_seed(seed, px, py);
  const Philox4 r = philox4x32_10(sy * g + sx, 0, 0, TAG_SCAN, static_cast<uint32_t>(ps),
                                  static_cast<uint32_t>(ps >> 32));
  const double gd = static_cast<double>(g);
  const double sub_x = (static_cast<double>(sx) + u24(r.v[0])) / gd;
  const double sub_y = (static_cast<double>(sy) + u24(r.v[1])) / gd;
  return v3((static_cast<double>(px) + sub_x) * pw, (static_cast<double>(py) + sub_y) * ph, z0);
}

int or_scan_ray_origins(const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg, uint64_t seed,
                        double* origins) {
  const uint32_t w = scfg->width_px, h = scfg->height_px;
  const uint32_t spp = std::max<uint32_t>(scfg->samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::round(std::sqrt(static_cast<double>(spp))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  const double pw = ecfg->width / static_cast<double>(w), ph = ecfg->height / static_cast<double>(h);
  for (uint32_t py = 0; py < h; ++py)
    for (uint32_t px = 0; px < w; ++px)
      for (uint32_t sy = 0; sy < g; ++sy)
        for (uint32_t sx = 0; sx < g; ++sx) {
          const V3 o = scan_origin(seed, px, py, sx, sy, g, pw, ph, ecfg->depth + 0.1);
          const size_t r = (static_cast<size_t>(py) * w + px) * a + sy * g + sx;
          origins[3 * r] = o.x;
          origins[3 * r + 1] = o.y;
          origins[3 * r + 2] = o.z;
        }
  return 0;
}

int or_scan(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
            uint64_t seed, int mode, int threads, const double* sigma_c, float* out,
            uint8_t* image8, double* T64, uint16_t* ray_hits_out) {
  const uint32_t w = scfg->width_px, h = scfg->height_px;
  const uint32_t spp = std::max<uint32_t>(scfg->samples_per_pixel, 1);
  const double pw = ecfg->width / static_cast<double>(w), ph = ecfg->height / static_cast<double>(h);
  std::vector<Crystal> dev;
  std::vector<size_t> orig;
  for (size_t i = 0; i < c->n; ++i) {
    Crystal k = load_crystal(c, i);
    if (k.developed) {
      dev.push_back(k);
      orig.push_back(i);
    }
  }
  RefBvh bvh;
  bvh.build(dev);
  const uint32_t g = static_cast<uint32_t>(std::round(std::sqrt(static_cast<double>(spp))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
  {
    std::vector<Hit> hits;
#pragma omp for schedule(dynamic, 1)
    for (int64_t py = 0; py < static_cast<int64_t>(h); ++py) {
      for (uint32_t px = 0; px < w; ++px) {
        double acc = 0.0;
        for (uint32_t sy = 0; sy < g; ++sy)
          for (uint32_t sx = 0; sx < g; ++sx) {
            const V3 o = scan_origin(seed, px, static_cast<uint32_t>(py), sx, sy, g, pw, ph,
                                     ecfg->depth + 0.1);
            double L = 0.0, tau = 0.0;
            size_t nh = 0;
            if (!dev.empty()) {
              ray_hits(bvh, dev, o, v3(0.0, 0.0, -1.0), mode, hits);
              for (const Hit& hh : hits) {
                const double chord = rmax(hh.t1 - hh.t0, 0.0);
                L += chord;
                if (sigma_c) tau += sigma_c[orig[hh.idx]] * chord;
              }
              nh = hits.size();
            }
            const double T = sigma_c ? std::exp(-tau) : std::exp(-scfg->silver_opacity * L);
            acc += T;
            if (ray_hits_out)
              ray_hits_out[(static_cast<size_t>(py) * w + px) * a + sy * g + sx] =
                  static_cast<uint16_t>(std::min<size_t>(nh, 65535));
          }
        const double mean64 = acc / static_cast<double>(a);
        const float mean = static_cast<float>(mean64);
        const size_t idx = static_cast<size_t>(py) * w + px;
        if (T64) T64[idx] = mean64;
        float v;
        if (scfg->mode == 0) {
          v = mean;
        } else if (scfg->mode == 1) {
          v = 1.0f - mean;
        } else {
          const float t = std::fmax(mean, 1e-4f);
          const float od = -std::log10(t);
          v = std::fmin(std::fmax(od / 3.0f, 0.0f), 1.0f);
        }
        out[idx] = v;
        if (image8) {
          const float cl = std::fmin(std::fmax(v, 0.0f), 1.0f);
          image8[idx] = static_cast<uint8_t>(std::round(cl * 255.0f));
        }
      }
    }
  }
  return 0;
}

// FP64 transmittance of pixel windows of a scan, each under +-hstep on one crystal's opacity (the
// reference's tree over all developed crystals, as or_scan builds it, built once).  Window k is
// win[4k..4k+3] = (x0, y0, w, h) in absolute pixels and perturbs crystal pidx[k]; T_out receives,
// window after window, three planes of w*h doubles: base, +hstep, -hstep.
int64_t or_scan_windows(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg, uint64_t seed,
                        int threads, const double* sigma_c, int64_t nwin, const uint32_t* win, const uint32_t* pidx,
                        double hstep, double* T_out) {
  const uint32_t W = scfg->width_px, H = scfg->height_px;
  const uint32_t spp = std::max<uint32_t>(scfg->samples_per_pixel, 1);
  const double pw = ecfg->width / static_cast<double>(W), ph = ecfg->height / static_cast<double>(H);
  std::vector<Crystal> dev;
  std::vector<size_t> orig;
  for (size_t i = 0; i < c->n; ++i) {
    Crystal k = load_crystal(c, i);
    if (k.developed) {
      dev.push_back(k);
      orig.push_back(i);
    }
  }
  RefBvh bvh;
  bvh.build(dev);
  const uint32_t g = static_cast<uint32_t>(std::round(std::sqrt(static_cast<double>(spp))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  const int nt = threads > 0 ? threads : omp_get_max_threads();
  size_t base = 0;
  for (int64_t k = 0; k < nwin; ++k) {
    const uint32_t x0 = win[4 * k], y0 = win[4 * k + 1], w = win[4 * k + 2], h = win[4 * k + 3];
    const size_t np = static_cast<size_t>(w) * h;
    double* tb = T_out + base;
    double* tp = tb + np;
    double* tm = tp + np;
#pragma omp parallel num_threads(nt)
    {
      std::vector<Hit> hits;
#pragma omp for schedule(dynamic, 1)
      for (int64_t yy = 0; yy < static_cast<int64_t>(h); ++yy) {
        for (uint32_t xx = 0; xx < w; ++xx) {
          const uint32_t px = x0 + xx, py = y0 + static_cast<uint32_t>(yy);
          double accb = 0.0, accp = 0.0, accm = 0.0;
          for (uint32_t sy = 0; sy < g; ++sy)
            for (uint32_t sx = 0; sx < g; ++sx) {
              double tau = 0.0, lc = 0.0;
              if (px < W && py < H && !dev.empty()) {
                const V3 o = scan_origin(seed, px, py, sx, sy, g, pw, ph, ecfg->depth + 0.1);
                ray_hits(bvh, dev, o, v3(0.0, 0.0, -1.0), OR_FAITHFUL, hits);
                for (const Hit& hh : hits) {
                  const double chord = rmax(hh.t1 - hh.t0, 0.0);
                  tau += (sigma_c ? sigma_c[orig[hh.idx]] : scfg->silver_opacity) * chord;
                  if (orig[hh.idx] == pidx[k]) lc += chord;
                }
              }
              accb += std::exp(-tau);
              accp += std::exp(-(tau + hstep * lc));
              accm += std::exp(-(tau - hstep * lc));
            }
          const size_t i = static_cast<size_t>(yy) * w + xx;
          tb[i] = accb / static_cast<double>(a);
          tp[i] = accp / static_cast<double>(a);
          tm[i] = accm / static_cast<double>(a);
        }
      }
    }
    base += 3 * np;
  }
  return static_cast<int64_t>(base);
}

// ---- differentiable scan and its adjoint (FP64) ----

void or_otf_taps(double s, double taps[3], double dtaps[3]) {
  // g = exp(-1 / (2 s^2)); taps = (g, 1, g) / (1 + 2 g); dg/ds = g / s^3.
  const double g = std::exp(-1.0 / (2.0 * s * s));
  const double n = 1.0 + 2.0 * g;
  taps[0] = taps[2] = g / n;
  taps[1] = 1.0 / n;
  const double dg = g / (s * s * s);
  dtaps[0] = dtaps[2] = dg / (n * n);
  dtaps[1] = -2.0 * dg / (n * n);
}

// One separable clamp-to-edge 3-tap pass (image_pipeline.rs:833-853) along x (axis 0) or y.
static void otf_pass(const double* in, uint32_t w, uint32_t h, const double k[3], int axis, double* out) {
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const size_t i = static_cast<size_t>(y) * w + x;
      size_t im, ip;
      if (axis == 0) {
        im = static_cast<size_t>(y) * w + (x > 0 ? x - 1 : 0);
        ip = static_cast<size_t>(y) * w + std::min(x + 1, w - 1);
      } else {
        im = static_cast<size_t>(y > 0 ? y - 1 : 0) * w + x;
        ip = static_cast<size_t>(std::min(y + 1, h - 1)) * w + x;
      }
      out[i] = in[im] * k[0] + in[i] * k[1] + in[ip] * k[2];
    }
}

// Transpose of otf_pass: scatters each output's weights back onto the pixels it read.
static void otf_pass_t(const double* g, uint32_t w, uint32_t h, const double k[3], int axis, double* out) {
  std::fill(out, out + static_cast<size_t>(w) * h, 0.0);
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const size_t i = static_cast<size_t>(y) * w + x;
      size_t im, ip;
      if (axis == 0) {
        im = static_cast<size_t>(y) * w + (x > 0 ? x - 1 : 0);
        ip = static_cast<size_t>(y) * w + std::min(x + 1, w - 1);
      } else {
        im = static_cast<size_t>(y > 0 ? y - 1 : 0) * w + x;
        ip = static_cast<size_t>(std::min(y + 1, h - 1)) * w + x;
      }
      out[im] += k[0] * g[i];
      out[i] += k[1] * g[i];
      out[ip] += k[2] * g[i];
    }
}

int or_scan_signal(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
                   uint64_t seed, int mode, int threads, const double* sigma_c, double exposure,
                   double otf_sigma, double* S, double* T) {
  const uint32_t w = scfg->width_px, h = scfg->height_px;
  const size_t np = static_cast<size_t>(w) * h;
  std::vector<float> out(np);
  std::vector<double> t64(np), tmp(np);
  or_scan_cfg cfg = *scfg;
  cfg.mode = 0;
  or_scan(c, ecfg, &cfg, seed, mode, threads, sigma_c, out.data(), nullptr, t64.data(), nullptr);
  double k[3], dk[3];
  or_otf_taps(otf_sigma, k, dk);
  otf_pass(t64.data(), w, h, k, 0, tmp.data());
  otf_pass(tmp.data(), w, h, k, 1, S);
  for (size_t i = 0; i < np; ++i) S[i] *= exposure;
  if (T) std::copy(t64.begin(), t64.end(), T);
  return 0;
}

int or_scan_backward(const or_crystals* c, const or_emulsion_cfg* ecfg, const or_scan_cfg* scfg,
                     uint64_t seed, int mode, int threads, const double* sigma_c, double exposure,
                     double otf_sigma, const double* dL_dS, double* g_sigma, double* g_exposure,
                     double* g_otf) {
  const uint32_t w = scfg->width_px, h = scfg->height_px;
  const size_t np = static_cast<size_t>(w) * h;
  const uint32_t spp = std::max<uint32_t>(scfg->samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::round(std::sqrt(static_cast<double>(spp))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  const double pw = ecfg->width / static_cast<double>(w), ph = ecfg->height / static_cast<double>(h);
  // Forward T, recomputed from the developed mask.
  std::vector<float> out(np);
  std::vector<double> T(np), H(np), dH(np), O(np), dO1(np), dO2(np), A1(np), A(np);
  or_scan_cfg cfg = *scfg;
  cfg.mode = 0;
  or_scan(c, ecfg, &cfg, seed, mode, threads, sigma_c, out.data(), nullptr, T.data(), nullptr);
  double k[3], dk[3];
  or_otf_taps(otf_sigma, k, dk);
  // S = e V(H(T)); dS/ds = e (V'(H(T)) + V(H'(T))); dS/de = V(H(T)).
  otf_pass(T.data(), w, h, k, 0, H.data());
  otf_pass(T.data(), w, h, dk, 0, dH.data());
  otf_pass(H.data(), w, h, k, 1, O.data());
  otf_pass(H.data(), w, h, dk, 1, dO1.data());
  otf_pass(dH.data(), w, h, k, 1, dO2.data());
  double ge = 0.0, gs = 0.0;
  for (size_t i = 0; i < np; ++i) {
    ge += dL_dS[i] * O[i];
    gs += dL_dS[i] * (dO1[i] + dO2[i]);
  }
  if (g_exposure) *g_exposure = ge;
  if (g_otf) *g_otf = exposure * gs;
  if (!g_sigma) return 0;
  // dL/dT = e H^T(V^T(dL/dS)); dT/dsigma_c = mean over the pixel's rays of -T_ray L_c.
  otf_pass_t(dL_dS, w, h, k, 1, A1.data());
  otf_pass_t(A1.data(), w, h, k, 0, A.data());
  std::fill(g_sigma, g_sigma + c->n, 0.0);
  std::vector<Crystal> dev;
  std::vector<size_t> orig;
  for (size_t i = 0; i < c->n; ++i) {
    Crystal kk = load_crystal(c, i);
    if (kk.developed) {
      dev.push_back(kk);
      orig.push_back(i);
    }
  }
  if (dev.empty()) return 0;
  RefBvh bvh;
  bvh.build(dev);
  const int nt = threads > 0 ? threads : omp_get_max_threads();
  std::vector<std::vector<double>> part(nt, std::vector<double>(c->n, 0.0));
#pragma omp parallel num_threads(nt)
  {
    std::vector<Hit> hits;
    std::vector<double>& gp = part[omp_get_thread_num()];
#pragma omp for schedule(static)
    for (int64_t py = 0; py < static_cast<int64_t>(h); ++py)
      for (uint32_t px = 0; px < w; ++px) {
        const double coef = -exposure * A[static_cast<size_t>(py) * w + px] / static_cast<double>(a);
        if (coef == 0.0) continue;
        for (uint32_t sy = 0; sy < g; ++sy)
          for (uint32_t sx = 0; sx < g; ++sx) {
            const V3 o = scan_origin(seed, px, static_cast<uint32_t>(py), sx, sy, g, pw, ph, ecfg->depth + 0.1);
            ray_hits(bvh, dev, o, v3(0.0, 0.0, -1.0), mode, hits);
            double tau = 0.0;
            for (const Hit& hh : hits)
              tau += (sigma_c ? sigma_c[orig[hh.idx]] : scfg->silver_opacity) * rmax(hh.t1 - hh.t0, 0.0);
            const double tr = std::exp(-tau);
            for (const Hit& hh : hits) gp[orig[hh.idx]] += coef * tr * rmax(hh.t1 - hh.t0, 0.0);
          }
      }
  }
  for (int t = 0; t < nt; ++t)
    for (size_t i = 0; i < c->n; ++i) g_sigma[i] += part[t][i];
  return 0;
}

// Preset tables for the tile worker (emulsion.rs:46-136, image_pipeline.rs:925-976).
static or_emulsion_cfg preset_cfg(int preset, double w, double h) {
  or_emulsion_cfg c{};
  c.width = w;
  c.height = h;
  c.optics.refractive_index = 1.534;
  if (preset == 0) {  // tri_x_400
    c.depth = 14.0; c.r_min = 1.2; c.mean_crystal_radius = 0.55; c.size_variance = 0.40;
    c.morphology = 0; c.tabular_aspect_ratio = 1.0;
    c.optics.absorption_coeff = 0.003; c.optics.scattering_coeff = 0.050; c.optics.anisotropy_g = 0.80;
    c.optics.antihalation_reflectance = 0.14; c.optics.antihalation_density = 0.80;
    c.base_sensitivity = 1.2;
  } else if (preset == 1) {  // tri_x_1600
    c.depth = 14.5; c.r_min = 1.1; c.mean_crystal_radius = 0.52; c.size_variance = 0.38;
    c.morphology = 0; c.tabular_aspect_ratio = 1.0;
    c.optics.absorption_coeff = 0.0032; c.optics.scattering_coeff = 0.052; c.optics.anisotropy_g = 0.80;
    c.optics.antihalation_reflectance = 0.14; c.optics.antihalation_density = 0.80;
    c.base_sensitivity = 1.35;
  } else if (preset == 2) {  // t_max_100
    c.depth = 8.0; c.r_min = 0.9; c.mean_crystal_radius = 0.40; c.size_variance = 0.20;
    c.morphology = 1; c.tabular_aspect_ratio = 6.5;
    c.optics.absorption_coeff = 0.002; c.optics.scattering_coeff = 0.035; c.optics.anisotropy_g = 0.85;
    c.optics.antihalation_reflectance = 0.08; c.optics.antihalation_density = 1.10;
    c.base_sensitivity = 0.8;
  } else {  // hp5_plus
    c.depth = 12.5; c.r_min = 1.1; c.mean_crystal_radius = 0.50; c.size_variance = 0.30;
    c.morphology = 2; c.tabular_aspect_ratio = 1.0;
    c.optics.absorption_coeff = 0.0025; c.optics.scattering_coeff = 0.045; c.optics.anisotropy_g = 0.82;
    c.optics.antihalation_reflectance = 0.12; c.optics.antihalation_density = 0.85;
    c.base_sensitivity = 1.1;
  }
  return c;
}

int or_render_tile(int preset, double pixel_size_um, const float* tile, uint32_t tw, uint32_t th,
                   double exposure, double push, uint64_t tile_seed, int mode, int threads,
                   float* d_neg, or_tile_report* rep) {
  // Effective push: the "1600" presets develop at least two stops (image_pipeline.rs:369-375).
  const double eff_push = preset == 1 ? rmax(push, 2.0) : rmax(push, 0.0);
  const double pw = static_cast<double>(tw) * pixel_size_um;
  const double ph = static_cast<double>(th) * pixel_size_um;
  int emul = preset;
  if (preset == 0 && eff_push >= 1.5) emul = 1;
  const or_emulsion_cfg ec = preset_cfg(emul, pw, ph);
  // Capacity from a loose bound on the packing density.
  const double vol = pw * ph * ec.depth;
  size_t cap = static_cast<size_t>(vol / (ec.r_min * ec.r_min * ec.r_min) * 1.2) + 64;
  std::vector<double> pos, dims, quat, sens, fe;
  std::vector<int32_t> morph;
  std::vector<uint32_t> lat;
  std::vector<uint8_t> dev;
  std::vector<int64_t> clump;
  or_crystals cr{};
  for (;;) {
    pos.assign(cap * 3, 0); dims.assign(cap * 3, 0); quat.assign(cap * 4, 0); sens.assign(cap, 0);
    morph.assign(cap, 0); lat.assign(cap, 0); dev.assign(cap, 0); clump.assign(cap, -1); fe.assign(cap, 1.0);
    cr = or_crystals{cap, pos.data(), dims.data(), quat.data(), sens.data(), morph.data(),
                     lat.data(), dev.data(), clump.data(), fe.data()};
    const int64_t n = or_synthesize(&ec, tile_seed, &cr);
    if (n <= static_cast<int64_t>(cap)) break;
    cap = static_cast<size_t>(n);
  }
  or_exposure_cfg xc{};
  xc.photons_per_sq_um = 6.0 * rmax(exposure, 0.05);
  xc.illumination_angle_rad = 0.12;
  xc.crystal_absorption_coeff = 1.3;
  xc.max_bounces = 48;
  uint64_t hits = 0;
  const int64_t P = or_expose(&cr, &ec, tile, tw, th, &xc, tile_seed + 1, mode, threads, nullptr, 0,
                              nullptr, &hits);
  or_dev_cfg dc{};
  dc.threshold_photons = 4;
  if (preset == 2) {
    dc.filament_expansion = 1.10 + 0.04 * eff_push;
    dc.clumping_proximity_factor = 1.10 + 0.03 * eff_push;
  } else if (preset == 3) {
    dc.filament_expansion = 1.15 + 0.05 * eff_push;
    dc.clumping_proximity_factor = 1.18 + 0.04 * eff_push;
  } else {
    dc.filament_expansion = 1.20 + 0.06 * eff_push;
    dc.clumping_proximity_factor = 1.25 + 0.05 * eff_push;
  }
  dc.developer_contrast = 0.85 + 0.05 * eff_push;
  or_dev_report dr;
  or_develop(&cr, &dc, &dr);
  or_scan_cfg sc{};
  sc.width_px = tw;
  sc.height_px = th;
  sc.samples_per_pixel = 4;
  sc.mode = 0;
  sc.silver_opacity = 0.25;
  std::vector<float> T(static_cast<size_t>(tw) * th);
  or_scan(&cr, &ec, &sc, tile_seed + 2, mode, threads, nullptr, T.data(), nullptr, nullptr, nullptr);
  for (size_t i = 0; i < T.size(); ++i) {
    const double t = rclamp(static_cast<double>(T[i]), 1e-4, 1.0);
    d_neg[i] = static_cast<float>(-std::log10(t) + 0.05);
  }
  if (rep) {
    rep->crystals = cr.n;
    rep->developed = dr.developed_crystals;
    rep->clumps = dr.total_clumps;
    rep->photons = static_cast<uint64_t>(P);
    rep->hits = hits;
  }
  return 0;
}

int or_scanner_otf(const float* in, uint32_t w, uint32_t h, const float k[3], float* out) {
  std::vector<float> tmp(static_cast<size_t>(w) * h);
  for (uint32_t y = 0; y < h; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      const uint32_t xm = x > 0 ? x - 1 : 0, xp = std::min(x + 1, w - 1);
      const size_t r = static_cast<size_t>(y) * w;
      tmp[r + x] = in[r + xm] * k[0] + in[r + x] * k[1] + in[r + xp] * k[2];
    }
  for (uint32_t y = 0; y < h; ++y) {
    const uint32_t ym = y > 0 ? y - 1 : 0, yp = std::min(y + 1, h - 1);
    for (uint32_t x = 0; x < w; ++x)
      out[static_cast<size_t>(y) * w + x] = tmp[static_cast<size_t>(ym) * w + x] * k[0] +
                                            tmp[static_cast<size_t>(y) * w + x] * k[1] +
                                            tmp[static_cast<size_t>(yp) * w + x] * k[2];
  }
  return 0;
}

// One separable pass of the tent-filter resampler along an axis of length n -> m.
static void tent_weights(uint32_t n, uint32_t m, std::vector<uint32_t>& left,
                         std::vector<uint32_t>& cnt, std::vector<float>& wts, uint32_t& stride) {
  const float ratio = static_cast<float>(n) / static_cast<float>(m);
  const float sratio = ratio < 1.0f ? 1.0f : ratio;
  const float support = 1.0f * sratio;
  stride = static_cast<uint32_t>(std::ceil(support * 2.0f)) + 2;
  left.assign(m, 0);
  cnt.assign(m, 0);
  wts.assign(static_cast<size_t>(m) * stride, 0.0f);
  for (uint32_t o = 0; o < m; ++o) {
    float in = (static_cast<float>(o) + 0.5f) * ratio;
    int64_t l = static_cast<int64_t>(std::floor(in - support));
    l = std::clamp<int64_t>(l, 0, static_cast<int64_t>(n) - 1);
    int64_t r = static_cast<int64_t>(std::ceil(in + support));
    r = std::clamp<int64_t>(r, l + 1, static_cast<int64_t>(n));
    in -= 0.5f;
    float sum = 0.0f;
    const uint32_t c = static_cast<uint32_t>(std::min<int64_t>(r - l, stride));
    for (uint32_t i = 0; i < c; ++i) {
      const float x = (static_cast<float>(l + i) - in) / sratio;
      const float ax = std::fabs(x);
      const float wv = ax < 1.0f ? 1.0f - ax : 0.0f;
      wts[static_cast<size_t>(o) * stride + i] = wv;
      sum += wv;
    }
    for (uint32_t i = 0; i < c; ++i) wts[static_cast<size_t>(o) * stride + i] /= sum;
    left[o] = static_cast<uint32_t>(l);
    cnt[o] = c;
  }
}

int or_resize_triangle(const float* in, uint32_t w, uint32_t h, uint32_t ow, uint32_t oh,
                       float* out) {
  // Vertical pass first, then horizontal (the order the image crate's resize uses).
  std::vector<uint32_t> l, c;
  std::vector<float> wt;
  uint32_t st;
  tent_weights(h, oh, l, c, wt, st);
  std::vector<float> tmp(static_cast<size_t>(w) * oh);
  for (uint32_t y = 0; y < oh; ++y)
    for (uint32_t x = 0; x < w; ++x) {
      float s = 0.0f;
      for (uint32_t i = 0; i < c[y]; ++i)
        s += wt[static_cast<size_t>(y) * st + i] * in[static_cast<size_t>(l[y] + i) * w + x];
      tmp[static_cast<size_t>(y) * w + x] = s;
    }
  tent_weights(w, ow, l, c, wt, st);
  for (uint32_t y = 0; y < oh; ++y)
    for (uint32_t x = 0; x < ow; ++x) {
      float s = 0.0f;
      for (uint32_t i = 0; i < c[x]; ++i)
        s += wt[static_cast<size_t>(x) * st + i] * tmp[static_cast<size_t>(y) * w + l[x] + i];
      out[static_cast<size_t>(y) * ow + x] = s;
    }
  return 0;
}

int or_blend_tiles(uint32_t out_w, uint32_t out_h, uint32_t tile_step, uint32_t pad,
                   uint32_t ntiles, const uint32_t* desc, const float* const* tiles,
                   float* d_norm) {
  const uint32_t ntx = (out_w + tile_step - 1) / tile_step, nty = (out_h + tile_step - 1) / tile_step;
  std::vector<float> acc(static_cast<size_t>(out_w) * out_h, 0.0f), wacc(acc.size(), 0.0f);
  const float pad2 = static_cast<float>(2 * pad);
  const float pi = 3.14159265358979323846f;
  auto hann = [&](uint32_t t, uint32_t g, uint32_t nt, uint32_t o0) {
    if (t > 0 && g < o0 + pad) {
      const float u = (static_cast<float>(g) - (static_cast<float>(o0) - static_cast<float>(pad))) / pad2;
      return 0.5f - 0.5f * std::cos(pi * std::fmin(std::fmax(u, 0.0f), 1.0f));
    }
    if (t + 1 < nt && g >= o0 + tile_step - pad) {
      const float u = (static_cast<float>(g) - (static_cast<float>(o0 + tile_step) - static_cast<float>(pad))) / pad2;
      return 0.5f + 0.5f * std::cos(pi * std::fmin(std::fmax(u, 0.0f), 1.0f));
    }
    return 1.0f;
  };
  for (uint32_t t = 0; t < ntiles; ++t) {
    const uint32_t tx = desc[6 * t], ty = desc[6 * t + 1], xs = desc[6 * t + 2], ys = desc[6 * t + 3];
    const uint32_t tw = desc[6 * t + 4], th = desc[6 * t + 5];
    const uint32_t x0 = tx * tile_step, y0 = ty * tile_step;
    for (uint32_t py = 0; py < th; ++py) {
      const uint32_t gy = ys + py;
      const float wy = hann(ty, gy, nty, y0);
      for (uint32_t px = 0; px < tw; ++px) {
        const uint32_t gx = xs + px;
        const float wv = hann(tx, gx, ntx, x0) * wy;
        const size_t gi = static_cast<size_t>(gy) * out_w + gx;
        acc[gi] += tiles[t][static_cast<size_t>(py) * tw + px] * wv;
        wacc[gi] += wv;
      }
    }
  }
  for (size_t i = 0; i < acc.size(); ++i) d_norm[i] = acc[i] / std::fmax(wacc[i], 1e-5f);
  return 0;
}

}  // extern "C"
