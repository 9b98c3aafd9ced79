// The reference's crystal BVH rebuilt on the device ("reference tree"): the same tree that
// BVH::build (bvh.rs:157-295) makes on the CPU, so that ray walks reach the same leaves and
// report crystals in the same order as BVH::intersect_ray_all (bvh.rs:300-347).
//
// The reference tree is a top-down spatial-median tree over the crystals' max_dim boxes
// (crystal.rs:106-133): a node of more than four crystals splits on the largest axis of its
// centroid box at the box's midpoint, unless that extent is at most 1e-7 (then it is a leaf).
// Which crystals a leaf holds, the boxes and the child order depend only on these sets; the order
// of the crystals inside a leaf is the result of the reference's in-place swap partition applied
// level after level, which the builder reproduces exactly (fg_rtree.cu).
//
// Why it matters: a leaf box is the union of its crystals' boxes, and the reference tests every
// crystal of every leaf whose box a ray hits by its geometry alone.  A rotated cube's corner
// sticks out of its own max_dim box by up to (sqrt(3) - 1) max_dim; the reference finds such a
// hit whenever the corner lies inside the leaf box.  And the transport absorbs hits in traversal
// order (right subtree first, leaf crystals in index order), which sets how the packet energy is
// shared between the crystals along a segment.
//
// Walk records.  Node ids are tile-local; the root is id 1, children come in pairs (l, l + 1) =
// (left, right).  The walks run over four-wide records: the record of an internal node at odd depth
// (the root's is record 0, any other's is record l / 2 of its children's pair l) holds that node's
// grandchildren, a leaf child taking one slot itself, in the order the reference's walk visits
// them (right subtree before left: RR, RL, LR, LL).  A child box contains its descendants' boxes,
// and the slab test is monotone in the box, so testing a grandchild alone reaches exactly the
// leaves the binary walk reaches, in the same order.  An internal child's FP32 box is its box
// rounded outward, padded, and extended by the crystals' reach beyond their own boxes, so that a
// walk clipped to a segment [0, step] still reaches every leaf holding a crystal the segment hits
// (the corner of a rotated cube can lie outside its leaf's box, nearer than the box); a leaf
// child's box is rounded to nearest, for the reference's own leaf test.
#pragma once
#include "fg_device.cuh"

namespace fg {

constexpr int RT_CTA_MAX = 1024;   // nodes of at most this many crystals are finished by one block
constexpr int RT_MAX_DEPTH = 47;   // deeper trees are rejected (bounds the walks' stacks)
constexpr int RT_STACK4 = 3 * ((RT_MAX_DEPTH + 1) / 2);  // four-wide walk: three pushes per record level
constexpr uint32_t RT_DONE = 0x80000000u;

// Per-tree input and bookkeeping of one tile (or one emulsion).  Element slots are tile-relative.
struct __align__(16) RTile {
  const float4* a;         // crystal records: position (xyz)
  const float4* d;         // half-dimensions (xyz)
  const double* pos64;     // FP64 copies (3 per slot) or null: then the FP32 records are exact
  const double* dims64;
  const double* exp64;     // expansion per slot (developed geometry) or null (1.0)
  const uint32_t* order;   // initial element order: order[k] - obase is element k's slot (null: k)
  unsigned long long obase;
  unsigned long long ebase;  // first element position of the tile
  unsigned long long nbase;  // first node of the tile
  uint32_t ecap, ncap;       // element and node capacity
  uint32_t n;                // elements (device-written before the build)
  uint32_t nodes;            // nodes made (written by the build)
  uint32_t depth;            // deepest level (written by the build)
  float pad;                 // outward padding of internal boxes in the FP32 walk records
  float reach;               // and their extension by the crystals' reach beyond their own boxes
  uint32_t rbase, rcap;      // first walk record of the tile, and the tile's record capacity
  uint32_t _pad;
};
static_assert(sizeof(RTile) == 112, "RTile layout");

// How far a crystal's geometry reaches beyond its own max_dim box (crystal.rs:106-217): a cube of
// half-size m lies within sqrt(3) m of its centre, an ellipsoid (the tabular and octahedral
// shapes) within m; so (sqrt(3) - 1) m for a set with cubes (m its largest half-size), else 0,
// plus a margin for FP32 rounding.
inline float rt_reach(double max_half_dim) {
  return static_cast<float>(0.7320508075688773 * max_half_dim * 1.0001 + 1e-5);
}

// Sizes of a one-tile build in caller-held memory (rtree_attach): nodes for ecap elements (at most
// 0.8 per element plus 64; the reference tree needs about 0.67), prefix-sum blocks, and the bytes
// of all buffers, each started on a 256-byte boundary (leafof: one word per crystal slot).
constexpr size_t rt_attach_nodes(size_t e1) {
  return e1 + 2 < (e1 * 4 + 4) / 5 + 64 ? e1 + 2 : (e1 * 4 + 4) / 5 + 64;
}
constexpr size_t rt_attach_blocks(size_t e1) { return (e1 + 1 + 2047) / 2048; }
constexpr size_t rt_al(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t rtree_attach_bytes(size_t ecap, bool want_leafof, size_t slots) {
  const size_t e1 = ecap > 0 ? ecap : 1, n1 = rt_attach_nodes(e1);
  return rt_al(112) + 4 * rt_al(4 * e1) + 2 * rt_al(24 * e1) + 2 * rt_al(4 * (e1 + 1)) + rt_al(4 * rt_attach_blocks(e1)) +
         3 * rt_al(4 * e1) + rt_al(48 * n1) + rt_al(48 * n1) + rt_al(4 * n1) + 4 * rt_al(4 * n1) + rt_al(4 * n1) + rt_al(8 * n1) +
         rt_al(8 * n1) + 4 * rt_al(4 * n1) + rt_al(16) + rt_al(128 * (n1 / 2 + 1)) + rt_al(8 * n1) +
         (want_leafof ? rt_al(4 * (slots > 0 ? slots : 1)) : 0);
}

// Max_dim box of element slot s (crystal.rs:106-133) in FP64, and its centroid (bvh.rs:74-80).
__device__ __forceinline__ void rt_box(const RTile& t, uint32_t s, double lo[3], double hi[3], double c[3]) {
  double p[3], dm;
  if (t.pos64) {
    p[0] = t.pos64[3 * s];
    p[1] = t.pos64[3 * s + 1];
    p[2] = t.pos64[3 * s + 2];
    dm = fmax(fmax(t.dims64[3 * s], t.dims64[3 * s + 1]), t.dims64[3 * s + 2]);
  } else {
    const float4 a = t.a[s], d = t.d[s];
    p[0] = a.x;
    p[1] = a.y;
    p[2] = a.z;
    dm = fmax(fmax(static_cast<double>(d.x), static_cast<double>(d.y)), static_cast<double>(d.z));
  }
  const double m = __dmul_rn(dm, t.exp64 ? t.exp64[s] : 1.0);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    lo[i] = __dsub_rn(p[i], m);
    hi[i] = __dadd_rn(p[i], m);
    c[i] = __dmul_rn(0.5, __dadd_rn(lo[i], hi[i]));
  }
}

// Position xyz and half-size m = max_dim * expansion of element slot s, in FP64 (crystal.rs:114-119).
__device__ __forceinline__ double4_32a rt_pm(const RTile& t, uint32_t s) {
  double4_32a v;
  double dm;
  if (t.pos64) {
    v.x = t.pos64[3 * s];
    v.y = t.pos64[3 * s + 1];
    v.z = t.pos64[3 * s + 2];
    dm = fmax(fmax(t.dims64[3 * s], t.dims64[3 * s + 1]), t.dims64[3 * s + 2]);
  } else {
    const float4 a = t.a[s], d = t.d[s];
    v.x = a.x;
    v.y = a.y;
    v.z = a.z;
    dm = fmax(fmax(static_cast<double>(d.x), static_cast<double>(d.y)), static_cast<double>(d.z));
  }
  v.w = __dmul_rn(dm, t.exp64 ? t.exp64[s] : 1.0);
  return v;
}

// The box p -+ m and its centroid 0.5 (lo + hi), as rt_box computes them.
__device__ __forceinline__ void rt_box_pm(const double4_32a& v, double lo[3], double hi[3], double c[3]) {
  const double p[3] = {v.x, v.y, v.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    lo[i] = __dsub_rn(p[i], v.w);
    hi[i] = __dadd_rn(p[i], v.w);
    c[i] = __dmul_rn(0.5, __dadd_rn(lo[i], hi[i]));
  }
}

// Every leaf of a tree whose box overlaps the query box [lo, hi], through the four-wide records
// (fn(local leaf id); the order of the calls is not the reference's, for order-free queries such
// as BVH::query_radius, bvh.rs:350-402).  A leaf is reached iff its box and its ancestors' boxes
// overlap the query, and ancestor boxes contain their descendants'.  nrec bounds the records.
template <class F>
__device__ __forceinline__ void rt_walk4_box(const Node4* __restrict__ rec, float3 lo, float3 hi, uint32_t nrec,
                                             uint32_t* err, F&& fn) {
  int stack[RT_STACK4];
  int sp = 0, cur = 0;
  for (;;) {
    if (!index_ok(static_cast<uint32_t>(cur) < nrec, err, SITE_NODE, static_cast<uint32_t>(cur), nrec)) break;
    const Node4* nd = rec + cur;
    const float4 lx = __ldg(&nd->lox), ly = __ldg(&nd->loy), lz = __ldg(&nd->loz);
    const float4 hx = __ldg(&nd->hix), hy = __ldg(&nd->hiy), hz = __ldg(&nd->hiz);
    const int4 rf = __ldg(&nd->ref);
    const float ax[4] = {lx.x, lx.y, lx.z, lx.w}, ay[4] = {ly.x, ly.y, ly.z, ly.w}, az[4] = {lz.x, lz.y, lz.z, lz.w};
    const float bx[4] = {hx.x, hx.y, hx.z, hx.w}, by[4] = {hy.x, hy.y, hy.z, hy.w}, bz[4] = {hz.x, hz.y, hz.z, hz.w};
    const int r[4] = {rf.x, rf.y, rf.z, rf.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (r[k] == INT32_MIN) continue;
      if (ax[k] <= hi.x && bx[k] >= lo.x && ay[k] <= hi.y && by[k] >= lo.y && az[k] <= hi.z && bz[k] >= lo.z) {
        if (r[k] < 0) {
          fn(static_cast<uint32_t>(~r[k]));
        } else if (sp < RT_STACK4) {
          stack[sp++] = r[k];
        } else {
          atomicOr(err, ERR_STACK_OVERFLOW);
        }
      }
    }
    if (sp == 0) break;
    cur = stack[--sp];
  }
}

// AABB::intersect_ray (bvh.rs:96-124) in FP64 with Rust's NaN-ignoring min / max.
__device__ __forceinline__ bool rt_box_hit64(const double* b, D3 o, D3 inv) {
  const double t1x = __dmul_rn(__dsub_rn(b[0], o.x), inv.x), t2x = __dmul_rn(__dsub_rn(b[3], o.x), inv.x);
  const double t1y = __dmul_rn(__dsub_rn(b[1], o.y), inv.y), t2y = __dmul_rn(__dsub_rn(b[4], o.y), inv.y);
  const double t1z = __dmul_rn(__dsub_rn(b[2], o.z), inv.z), t2z = __dmul_rn(__dsub_rn(b[5], o.z), inv.z);
  const double te = fmax(fmax(fmin(t1x, t2x), fmin(t1y, t2y)), fmin(t1z, t2z));
  const double tx = fmin(fmin(fmax(t1x, t2x), fmax(t1y, t2y)), fmax(t1z, t2z));
  return tx >= te && tx > 0.0;
}

// The reference walk, exactly (bvh.rs:300-347): pop a node, test its box on the whole ray in
// FP64, call fn(leaf id) for a leaf, else push left then right when fewer than 62 entries are on
// the stack (more are dropped, as the reference drops them).  nodes / box64 / nchild are the
// tile's build arrays (global ids, nbase applied by the caller).
template <class F>
__device__ __forceinline__ void rt_walk64(const double* __restrict__ box64, const int2* __restrict__ nchild,
                                          const int* __restrict__ nsplit, uint32_t root, D3 o, D3 inv, F&& fn) {
  uint32_t stack[64];
  int sp = 0;
  stack[sp++] = root;
  while (sp > 0) {
    const uint32_t id = stack[--sp];
    if (!rt_box_hit64(box64 + 6 * static_cast<size_t>(id), o, inv)) continue;
    if (nsplit[id] < 0) {
      fn(id);
    } else if (sp + 2 < 64) {
      const int2 ch = nchild[id];
      stack[sp] = static_cast<uint32_t>(ch.x);
      stack[sp + 1] = static_cast<uint32_t>(ch.y);
      sp += 2;
    }
  }
}

}  // namespace fg
