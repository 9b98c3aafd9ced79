// Device-side building blocks shared by the fgrain GB300 kernels: Philox streams, the exact
// FP64 predicates of the reference, FP32 geometry, and the node / crystal layouts in HBM.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fg {

// ---------------------------------------------------------------------------------------------
// Philox-4x32-10 (Salmon et al., SC'11).  The stream of each draw is named by its counter:
// (photon id, bounce, slot, tag) for transport, (stratum, 0, 0, tag) under a per-pixel key for
// the scanner.  Uniforms keep 24 bits so float and double see the same value.
struct P4 {
  uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ P4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    const uint64_t m0 = (uint64_t)0xD2511F53u * c0, m1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(m0 >> 32), lo0 = (uint32_t)m0;
    const uint32_t hi1 = (uint32_t)(m1 >> 32), lo1 = (uint32_t)m1;
#endif
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return P4{c0, c1, c2, c3};
}

__host__ __device__ __forceinline__ float uf(uint32_t v) { return (float)(v >> 8) * 5.9604644775390625e-8f; }
__host__ __device__ __forceinline__ double ud(uint32_t v) { return (double)(v >> 8) * 5.9604644775390625e-8; }
__host__ __device__ __forceinline__ uint32_t word(const P4& p, uint32_t i) {
  return i == 0 ? p.x : (i == 1 ? p.y : (i == 2 ? p.z : p.w));
}

enum : uint32_t {
  TAG_EMIT = 0x454D0000u,
  TAG_BOUNCE = 0x424F0000u,
  TAG_AH = 0x41480000u,
  TAG_HIT = 0x48490000u,
  TAG_SCAN = 0x53430000u,
  TAG_DART = 0x44410000u,
  TAG_ATTR = 0x41540000u,
};

// ---------------------------------------------------------------------------------------------
// Layouts in HBM.
//
// Crystals are stored in Morton order (index s), structure-of-arrays, 48 bytes hot:
//   a[s] = (x, y, z, sensitivity)   q[s] = (qi, qj, qk, qw)   d[s] = (dx, dy, dz, morphology bits)
// The FP64 copy (pos, dims, quat) is present only for crystal sets uploaded from the host; a
// synthesized set is defined by its FP32 values, which double represents exactly.
struct CrystalsView {
  const float4* a;
  const float4* q;
  const float4* d;
  const double* pos64;   // 3 per crystal, or null
  const double* dims64;  // 3 per crystal, or null
  const double* quat64;  // 4 per crystal, or null
  const double* sens64;  // 1 per crystal, or null
  uint32_t n;
};

// Walk record: a four-wide node of the reference tree, 128 bytes.  Child k's FP32 box is
// (lox[k], loy[k], loz[k]) - (hix[k], hiy[k], hiz[k]); ref[k] is another record (its index, >= 0),
// a leaf (~tile-local node id, < 0) or empty (INT32_MIN).  Children are in visiting order.
struct __align__(16) Node4 {
  float4 lox, loy, loz, hix, hiy, hiz;
  int4 ref;
  int4 _pad;
};

__device__ __forceinline__ int morph_of(const float4& d) { return __float_as_int(d.w); }

// ---------------------------------------------------------------------------------------------
// Exact FP64 restatement of the reference predicates (crystal.rs:106-217, bvh.rs:96-124).
// Every operation is an explicitly rounded intrinsic so nvcc cannot fuse it; the CPU oracle is
// compiled with -ffp-contract=off, so both sides round identically.
struct D3 {
  double x, y, z;
};

__device__ __forceinline__ D3 d3(double x, double y, double z) { return D3{x, y, z}; }
__device__ __forceinline__ D3 dsub3(D3 a, D3 b) {
  return d3(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z));
}
__device__ __forceinline__ D3 dcross(D3 a, D3 b) {
  return d3(__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)),
            __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
            __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double ddot(D3 a, D3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
// UnitQuaternion::inverse_transform_vector: v + w t + q' x t, t = 2 (q' x v), q' conjugated.
__device__ __forceinline__ D3 dquat_inv_rotate(const double q[4], D3 v) {
  const D3 qv = d3(-q[0], -q[1], -q[2]);
  const D3 c1 = dcross(qv, v);
  const D3 t = d3(__dmul_rn(c1.x, 2.0), __dmul_rn(c1.y, 2.0), __dmul_rn(c1.z, 2.0));
  const D3 c2 = dcross(qv, t);
  return d3(__dadd_rn(__dadd_rn(__dmul_rn(t.x, q[3]), c2.x), v.x),
            __dadd_rn(__dadd_rn(__dmul_rn(t.y, q[3]), c2.y), v.y),
            __dadd_rn(__dadd_rn(__dmul_rn(t.z, q[3]), c2.z), v.z));
}

struct Crystal64 {
  D3 pos, dims;
  double q[4];
  double sens;
  int morph;
};

__device__ __forceinline__ Crystal64 load64(const CrystalsView& c, uint32_t s) {
  Crystal64 k;
  const float4 d = c.d[s];
  k.morph = morph_of(d);
  if (c.pos64) {
    k.pos = d3(c.pos64[3 * s], c.pos64[3 * s + 1], c.pos64[3 * s + 2]);
    k.dims = d3(c.dims64[3 * s], c.dims64[3 * s + 1], c.dims64[3 * s + 2]);
#pragma unroll
    for (int j = 0; j < 4; ++j) k.q[j] = c.quat64[4 * s + j];
    k.sens = c.sens64[s];
  } else {
    const float4 a = c.a[s], q = c.q[s];
    k.pos = d3(a.x, a.y, a.z);
    k.dims = d3(d.x, d.y, d.z);
    k.q[0] = q.x; k.q[1] = q.y; k.q[2] = q.z; k.q[3] = q.w;
    k.sens = a.w;
  }
  return k;
}

// max_dim * expansion (crystal.rs:114-119).
__device__ __forceinline__ double dmaxdim(const Crystal64& k, double e) {
  return __dmul_rn(fmax(fmax(k.dims.x, k.dims.y), k.dims.z), e);
}

// AABB::intersect_ray against the crystal's own box of half-side m (bvh.rs:96-124).
__device__ __forceinline__ bool dbox_hit(const Crystal64& k, double m, D3 o, D3 inv) {
  const double lx = __dsub_rn(k.pos.x, m), hx = __dadd_rn(k.pos.x, m);
  const double ly = __dsub_rn(k.pos.y, m), hy = __dadd_rn(k.pos.y, m);
  const double lz = __dsub_rn(k.pos.z, m), hz = __dadd_rn(k.pos.z, m);
  const double t1x = __dmul_rn(__dsub_rn(lx, o.x), inv.x), t2x = __dmul_rn(__dsub_rn(hx, o.x), inv.x);
  const double t1y = __dmul_rn(__dsub_rn(ly, o.y), inv.y), t2y = __dmul_rn(__dsub_rn(hy, o.y), inv.y);
  const double t1z = __dmul_rn(__dsub_rn(lz, o.z), inv.z), t2z = __dmul_rn(__dsub_rn(hz, o.z), inv.z);
  const double te = fmax(fmax(fmin(t1x, t2x), fmin(t1y, t2y)), fmin(t1z, t2z));
  const double tx = fmin(fmin(fmax(t1x, t2x), fmax(t1y, t2y)), fmax(t1z, t2z));
  return tx >= te && tx > 0.0;
}

// HalideCrystal::intersect_ray with expansion e (crystal.rs:140-217).
__device__ __forceinline__ bool dintersect(const Crystal64& k, double e, D3 o, D3 d, double& t0,
                                           double& t1) {
  const D3 lo = dquat_inv_rotate(k.q, dsub3(o, k.pos));
  const D3 ld = dquat_inv_rotate(k.q, d);
  const D3 dm = d3(__dmul_rn(k.dims.x, e), __dmul_rn(k.dims.y, e), __dmul_rn(k.dims.z, e));
  if (k.morph == 0) {
    const double ix = __ddiv_rn(1.0, ld.x), iy = __ddiv_rn(1.0, ld.y), iz = __ddiv_rn(1.0, ld.z);
    const double a1 = __dmul_rn(__dsub_rn(-dm.x, lo.x), ix), a2 = __dmul_rn(__dsub_rn(dm.x, lo.x), ix);
    const double b1 = __dmul_rn(__dsub_rn(-dm.y, lo.y), iy), b2 = __dmul_rn(__dsub_rn(dm.y, lo.y), iy);
    const double c1 = __dmul_rn(__dsub_rn(-dm.z, lo.z), iz), c2 = __dmul_rn(__dsub_rn(dm.z, lo.z), iz);
    const double tmin = fmax(fmax(fmin(a1, a2), fmin(b1, b2)), fmin(c1, c2));
    const double tmax = fmin(fmin(fmax(a1, a2), fmax(b1, b2)), fmax(c1, c2));
    if (tmax >= tmin && tmax > 0.0) {
      t0 = fmax(tmin, 0.0);
      t1 = tmax;
      return true;
    }
    return false;
  }
  const D3 p = d3(__ddiv_rn(lo.x, dm.x), __ddiv_rn(lo.y, dm.y), __ddiv_rn(lo.z, dm.z));
  const D3 dd = d3(__ddiv_rn(ld.x, dm.x), __ddiv_rn(ld.y, dm.y), __ddiv_rn(ld.z, dm.z));
  const double a = ddot(dd, dd);
  const double b = __dmul_rn(2.0, ddot(p, dd));
  const double c = __dsub_rn(ddot(p, p), 1.0);
  const double disc = __dsub_rn(__dmul_rn(b, b), __dmul_rn(__dmul_rn(4.0, a), c));
  if (disc < 0.0) return false;
  const double sq = __dsqrt_rn(disc);
  const double den = __dmul_rn(2.0, a);
  const double r0 = __ddiv_rn(__dsub_rn(-b, sq), den);
  const double r1 = __ddiv_rn(__dadd_rn(-b, sq), den);
  const double te = fmin(r0, r1), tx = fmax(r0, r1);
  if (tx > 0.0) {
    t0 = fmax(te, 0.0);
    t1 = tx;
    return true;
  }
  return false;
}

// Canonical hit: geometry hit and own max_dim box hit.
__device__ __forceinline__ bool dcanonical_hit(const Crystal64& k, double e, D3 o, D3 d, D3 inv,
                                               double& t0, double& t1) {
  if (!dintersect(k, e, o, d, t0, t1)) return false;
  return dbox_hit(k, dmaxdim(k, e), o, inv);
}

// ---------------------------------------------------------------------------------------------
// FP32 geometry.
__device__ __forceinline__ float3 quat_inv_rotate(float4 q, float3 v) {
  // t = 2 (q' x v), v' = v + w t + q' x t, q' = -q.xyz
  const float qx = -q.x, qy = -q.y, qz = -q.z;
  const float tx = 2.0f * (qy * v.z - qz * v.y);
  const float ty = 2.0f * (qz * v.x - qx * v.z);
  const float tz = 2.0f * (qx * v.y - qy * v.x);
  return make_float3(v.x + q.w * tx + (qy * tz - qz * ty), v.y + q.w * ty + (qz * tx - qx * tz),
                     v.z + q.w * tz + (qx * ty - qy * tx));
}

// Slab test of a ray against a box; returns entry/exit (not clamped).
__device__ __forceinline__ void slab(float3 o, float3 inv, float lx, float ly, float lz, float hx,
                                     float hy, float hz, float& te, float& tx) {
  const float t1x = (lx - o.x) * inv.x, t2x = (hx - o.x) * inv.x;
  const float t1y = (ly - o.y) * inv.y, t2y = (hy - o.y) * inv.y;
  const float t1z = (lz - o.z) * inv.z, t2z = (hz - o.z) * inv.z;
  te = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fminf(t1z, t2z));
  tx = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fmaxf(t1z, t2z));
}

// FP32 crystal geometry of a general ray (production transport), HalideCrystal::intersect_ray
// (crystal.rs:140-217): the oriented cube's slabs or the ellipsoid's quadratic, nothing else.
__device__ __forceinline__ bool fintersect(float4 a, float4 q, float4 d, float e, float3 o, float3 dir, float& t0,
                                           float& t1) {
  const float3 lo = quat_inv_rotate(q, make_float3(o.x - a.x, o.y - a.y, o.z - a.z));
  const float3 ld = quat_inv_rotate(q, dir);
  const float dx = d.x * e, dy = d.y * e, dz = d.z * e;
  if (morph_of(d) == 0) {
    const float ix = 1.0f / ld.x, iy = 1.0f / ld.y, iz = 1.0f / ld.z;
    const float a1 = (-dx - lo.x) * ix, a2 = (dx - lo.x) * ix;
    const float b1 = (-dy - lo.y) * iy, b2 = (dy - lo.y) * iy;
    const float c1 = (-dz - lo.z) * iz, c2 = (dz - lo.z) * iz;
    const float tmin = fmaxf(fmaxf(fminf(a1, a2), fminf(b1, b2)), fminf(c1, c2));
    const float tmax = fminf(fminf(fmaxf(a1, a2), fmaxf(b1, b2)), fmaxf(c1, c2));
    if (tmax >= tmin && tmax > 0.0f) {
      t0 = fmaxf(tmin, 0.0f);
      t1 = tmax;
      return true;
    }
    return false;
  }
  const float px = lo.x / dx, py = lo.y / dy, pz = lo.z / dz;
  const float ex = ld.x / dx, ey = ld.y / dy, ez = ld.z / dz;
  const float A = ex * ex + ey * ey + ez * ez;
  const float B = 2.0f * (px * ex + py * ey + pz * ez);
  const float C = px * px + py * py + pz * pz - 1.0f;
  const float disc = B * B - 4.0f * A * C;
  if (disc < 0.0f) return false;
  const float sq = sqrtf(disc);
  const float r0 = (-B - sq) / (2.0f * A), r1 = (-B + sq) / (2.0f * A);
  if (r1 > 0.0f) {
    t0 = fmaxf(r0, 0.0f);
    t1 = r1;
    return true;
  }
  return false;
}

// FP32 canonical hit: the crystal's own max_dim box and its geometry.
__device__ __forceinline__ bool fcanonical_hit(float4 a, float4 q, float4 d, float e, float3 o,
                                               float3 dir, float3 inv, float& t0, float& t1) {
  const float m = fmaxf(fmaxf(d.x, d.y), d.z) * e;
  float be, bx;
  slab(o, inv, a.x - m, a.y - m, a.z - m, a.x + m, a.y + m, a.z + m, be, bx);
  if (!(bx >= be && bx > 0.0f)) return false;
  return fintersect(a, q, d, e, o, dir, t0, t1);
}

// 2D Morton interleave of 16-bit coordinates.
__host__ __device__ inline uint32_t morton2_spread(uint32_t v) {
  v &= 0xffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
__host__ __device__ inline uint32_t morton2_compact(uint32_t v) {
  v &= 0x55555555u;
  v = (v | (v >> 1)) & 0x33333333u;
  v = (v | (v >> 2)) & 0x0f0f0f0fu;
  v = (v | (v >> 4)) & 0x00ff00ffu;
  v = (v | (v >> 8)) & 0x0000ffffu;
  return v;
}
// Every third bit of v from bit 0 (the inverse of a 3D Morton interleave, 10 bits out).
__host__ __device__ inline uint32_t morton3_compact(uint32_t v) {
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030c30c3u;
  v = (v | (v >> 4)) & 0x0300f00fu;
  v = (v | (v >> 8)) & 0x030000ffu;
  v = (v | (v >> 16)) & 0x000003ffu;
  return v;
}

// Error word bits written by kernels (read back by the host after each call).  The error record
// is four words: the bits, then (for ERR_BAD_INDEX) the site and two values of the first failed
// index check.
enum : uint32_t {
  ERR_HIT_OVERFLOW = 1u << 0,
  ERR_STACK_OVERFLOW = 1u << 1,
  ERR_SPIN_LIMIT = 1u << 2,
  ERR_LIST_OVERFLOW = 1u << 3,
  ERR_BAD_INPUT = 1u << 4,
  ERR_BAD_INDEX = 1u << 5,
};
constexpr int ERR_WORDS = 4;

// Sites of index checks (the second word of the error record).
enum : uint32_t {
  SITE_SYN_REGION = 1,   // synthesis: candidate neighbourhood outside the staged region
  SITE_SYN_COMMIT = 2,   // synthesis: accepted point outside the staged region
  SITE_SYN_ACTIVE = 3,   // synthesis: active list full
  SITE_PHOTON_CELL = 4,  // photon ordering: emission cell out of range
  SITE_PHOTON_SLOT = 5,  // photon ordering: slot past the photon count
  SITE_PHOTON_ID = 6,    // transport: ordered photon id past the photon count
  SITE_NODE = 7,         // tree walk: record index out of range
  SITE_LEAF = 8,         // tree walk: leaf id or its element range out of range
};

__device__ __noinline__ static void record_bad_index(uint32_t* err, uint32_t site, uint32_t a, uint32_t b) {
  atomicOr(err, ERR_BAD_INDEX);
  if (atomicCAS(err + 1, 0u, site) == 0u) {
    err[2] = a;
    err[3] = b;
  }
}

// Guard of an index computed from data: on failure the access is to be skipped and the failure is
// recorded in the error record.
__device__ __forceinline__ bool index_ok(bool ok, uint32_t* err, uint32_t site, uint32_t a, uint32_t b) {
  if (!ok) record_bad_index(err, site, a, b);
  return ok;
}

}  // namespace fg
