// Device code of the photon transport: tile descriptors, the reference-tree walk and the
// per-photon bounce loop (transport.rs:101-185, optics.rs:100-196).
#pragma once
#include "fg_device.cuh"
#include "fg_rtree.cuh"

namespace fg {

constexpr int WALK_LEAVES = 6;    // leaves a lane may hold while its warp still walks (speculative traversal)
constexpr int WALK_RESTART = 24;  // idle lanes of a warp that end and start their bounces together
constexpr int WALK_EMPTY = INT32_MIN;
constexpr uint32_t WALK_NONE = 0xffffffffu;

// Everything one tile's transport needs, 16-byte aligned for vector loads.  The walk runs over the
// tile's reference tree (fg_rtree.cuh): rnode / rleaf indexed by tile-local node id, ridx by
// tile-local element position (a leaf's crystals in the reference's order).  The crystal records
// a, q, d are in that element order too (position p holds the crystal ridx[p]), so a leaf's
// crystals lie next to each other and are read without their slots.
struct __align__(16) TileDesc {
  const float4* a;
  const float4* q;
  const float4* d;
  const Node4* rnode;     // four-wide walk records of the tile's tree
  const uint2* rleaf;
  const uint32_t* ridx;
  const uint32_t* s2id;
  uint32_t* counts;
  const float* tile;
  unsigned long long photon_base;
  uint32_t n, tw, th, P;
  uint32_t nnodes;  // node capacity of the tile's tree (bounds the leaf ids the walk reads)
  uint32_t nrec;    // walk records of the tile's tree (bounds the record indices)
  float reach;      // crystals' reach beyond their own boxes (fg_rtree.cuh)
  uint32_t stride;  // exposure row stride (floats); tiles may be windows of one image
  uint32_t pcell_base;  // first photon-sort cell of this tile
  uint32_t pcell_bits;  // photon-sort cells per axis = 2^bits (Morton order)
  float W, H, D;
  uint32_t k0, k1;
  float mu_t, albedo, g, r0, eff_r, theta_max, alpha;
  uint32_t max_bounces;
};

// 1 / d for the walk's slab tests, kept finite: the test forms lo * inv - o * inv with one FMA, and
// an infinite inv (a direction component of 0, or below 1e-30) would turn that into inf - inf =
// NaN, which fminf / fmaxf drop, so the axis would not constrain the box at all (a parent box
// could fail while its child passes).  With |inv| capped at 1e30 the products stay finite
// (coordinates are below 1e4 um) and the slab is (-huge, huge) or empty as for the reference's
// infinite inv (bvh.rs:96-124); only a box face within about 1e-7 relative of the ray's
// coordinate can be judged either way.
__device__ __forceinline__ float slab_inv(float d) {
  return fabsf(d) < 1e-30f ? copysignf(1e30f, d) : 1.0f / d;
}

// Beer-Lambert absorption of one hit and Bernoulli rounding of the latent photons
// (transport.rs:359-381), in exactly rounded FP64.
__device__ __forceinline__ double absorb64(double E, double path, double alpha, double sens,
                                           double u, uint32_t* count) {
  const double p = __dsub_rn(1.0, exp(__dmul_rn(-alpha, path)));
  const double absorbed = __dmul_rn(__dmul_rn(E, p), sens);
  const double expected = __dmul_rn(absorbed, 5.0);
  const double fl = floor(expected);
  const uint32_t whole = fl <= 0.0 ? 0u : (fl >= 4294967295.0 ? 4294967295u : static_cast<uint32_t>(fl));
  const double frac = __dsub_rn(expected, static_cast<double>(whole));
  *count = whole + ((u < fmin(fmax(frac, 0.0), 1.0)) ? 1u : 0u);
  return __dmul_rn(E, fmax(__dsub_rn(1.0, __dmul_rn(p, 0.9)), 0.05));
}

// Adds n latent photons to crystal s, one atomic per distinct counter among the active lanes.
// Lanes are grouped by the counter's address, not by s: the lanes of a warp may trace photons of
// different tiles, whose crystals share local indices.
__device__ __forceinline__ void add_counts(uint32_t* counts, uint32_t s, uint32_t n) {
  uint32_t* const ctr = counts + s;
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, reinterpret_cast<unsigned long long>(ctr));
  const int leader = __ffs(grp) - 1;
  uint32_t sum = 0;
  for (unsigned m = grp; m; m &= m - 1) sum += __shfl_sync(grp, n, __ffs(m) - 1);
  if ((threadIdx.x & 31) == leader && sum) atomicAdd(ctr, sum);
}

// ---------------------------------------------------------------------------------------------
// A packet between bounces (transport.rs:72-185): position, direction, energy, photon id and the
// number of bounces begun.  The transport kernel keeps one per lane and refills a lane whose packet
// died with the next photon while the rest of the warp carries on.
struct Photon {
  float3 pos, dir;
  float E;
  uint32_t id, b;
};

constexpr float PHOTON_CELL_UM = 1.0f;  // emission cells used to order photons

// Emission of photon `id` (transport.rs:72-97 with the tile worker's exposure closure).  Returns
// false when the packet never enters the gelatin (zero exposure, Fresnel reflection).
__device__ __forceinline__ bool emit_photon(const TileDesc& t, uint32_t id, Photon& ph) {
  const float PI2 = 6.283185307179586f;
  const P4 e0 = philox(id, 0, 0, TAG_EMIT, t.k0, t.k1);
  const float x = uf(e0.x) * t.W;
  const float y = uf(e0.y) * t.H;
  const float uu = fminf(fmaxf(x / t.W, 0.0f), 1.0f), vv = fminf(fmaxf(y / t.H, 0.0f), 1.0f);
  const uint32_t px = min(static_cast<uint32_t>(roundf(uu * (float)(t.tw - 1))), t.tw - 1);
  const uint32_t py = min(static_cast<uint32_t>(roundf(vv * (float)(t.th - 1))), t.th - 1);
  const float E = fmaxf(__ldg(&t.tile[static_cast<size_t>(py) * t.stride + px]), 0.0f);
  if (!(E > 0.0f)) return false;
  const float theta = uf(e0.z) * t.theta_max;
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(uf(e0.w) * PI2, &sp, &cp);
  float3 dir = make_float3(st * cp, st * sp, ct);
  const float n = rsqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
  dir = make_float3(dir.x * n, dir.y * n, dir.z * n);
  const float c = fminf(fabsf(dir.z), 1.0f), m = 1.0f - c, m2 = m * m;
  const float R = t.r0 + (1.0f - t.r0) * (m2 * m2 * m);
  if (uf(philox(id, 0, 1, TAG_EMIT, t.k0, t.k1).x) < R) return false;
  ph.pos = make_float3(x, y, 0.001f);
  ph.dir = dir;
  ph.E = E;
  ph.id = id;
  ph.b = 0;
  return true;
}

// One lane's bounce in progress (transport.rs:101-185): its segment, the packet's absorption so
// far and its walk of the tile's reference tree (the walk stack is the caller's).
//
// The walk follows the reference's order (BVH::intersect_ray_all, bvh.rs:300-347: push left then
// right, pop right first) over the four-wide records (fg_rtree.cuh), whose children are stored in
// that visiting order: the first hit child is entered, the other hit children are pushed so that
// they come off the stack in order.  An internal child is entered when its (extended) box meets
// [0, tlim] of the ray (the step, padded); a leaf child when its box extended by `reach` meets
// [0, tlim] (a crystal hit inside the step lies there) and its own box meets the whole ray (the
// reference's leaf test, bvh.rs:96-124).  Leaves are queued in walk order and tested later, so
// that a warp's lanes test leaves together (deferred, speculative traversal): a lane walks on
// while its queue has room.
struct Bounce {
  float3 inv, oi;     // 1 / dir (slab_inv) and pos * inv, for the slab tests
  float step, tlim;   // the step and the walk's reach along the ray
  float E;            // packet energy, as the hits absorb it
  uint32_t nh;        // absorbing hits so far
  P4 r;               // the Philox block of hits nh & ~3 .. (nh & ~3) + 3
  int cur, sp;        // current record (~leaf for a leaf child, WALK_EMPTY when done) and stack depth
  uint32_t lv[WALK_LEAVES];  // leaves reached and not yet tested, in walk order
};

// Starts bounce ph.b (transport.rs:101-107): the free path, the segment's step and the walk from
// the root record.
__device__ __forceinline__ void bounce_begin(const TileDesc& t, Photon& ph, Bounce& w) {
  const uint32_t b = ph.b++;
  const P4 rb = philox(ph.id, b, 0, TAG_BOUNCE, t.k0, t.k1);
  const float fp = t.mu_t > 0.0f ? -__logf(fmaxf(1.0f - uf(rb.x), 1.17549435e-38f)) / t.mu_t : 1e6f;
  w.step = fminf(fp, t.D * 1.5f);
  w.inv = make_float3(slab_inv(ph.dir.x), slab_inv(ph.dir.y), slab_inv(ph.dir.z));
  w.oi = make_float3(ph.pos.x * w.inv.x, ph.pos.y * w.inv.y, ph.pos.z * w.inv.z);
  w.tlim = w.step * 1.00001f + 1e-3f;
  w.E = ph.E;
  w.nh = 0;
  w.r = P4{};
  w.cur = 0;  // record 0: the root's
  w.sp = 0;
#pragma unroll
  for (int j = 0; j < WALK_LEAVES; ++j) w.lv[j] = WALK_NONE;
}

// One step of the walk: queue the leaf child taken last, or test the current record's four
// children (enter the first hit, push the later ones).  Only for a lane whose walk goes on
// (cur != WALK_EMPTY) and whose leaf queue has room.
__device__ __forceinline__ void walk_step(const TileDesc& t, Bounce& w, int* stack, uint32_t* err) {
  if (w.cur < 0) {
    const uint32_t lf = static_cast<uint32_t>(~w.cur);
    bool placed = false;
#pragma unroll
    for (int j = 0; j < WALK_LEAVES; ++j) {
      if (!placed && w.lv[j] == WALK_NONE) {
        w.lv[j] = lf;
        placed = true;
      }
    }
    w.cur = w.sp > 0 ? stack[--w.sp] : WALK_EMPTY;
    return;
  }
  if (!index_ok(static_cast<uint32_t>(w.cur) < t.nrec, err, SITE_NODE, static_cast<uint32_t>(w.cur), t.nrec)) {
    w.cur = WALK_EMPTY;
    return;
  }
  const Node4* nd = t.rnode + w.cur;
  const float4 lx = __ldg(&nd->lox), ly = __ldg(&nd->loy), lz = __ldg(&nd->loz);
  const float4 hx = __ldg(&nd->hix), hy = __ldg(&nd->hiy), hz = __ldg(&nd->hiz);
  const int4 rf = __ldg(&nd->ref);
  const float3 inv = w.inv, oi = w.oi;
  const float tlim = w.tlim, reach = t.reach;
  // Slab test as lo * inv - o * inv (one FMA per plane), the box grown by g, clipped to [0, tm].
  auto slab_hit = [&](float a0, float a1, float a2, float a3, float a4, float a5, float g, float tm) {
    const float t1x = fmaf(a0 - g, inv.x, -oi.x), t2x = fmaf(a3 + g, inv.x, -oi.x);
    const float t1y = fmaf(a1 - g, inv.y, -oi.y), t2y = fmaf(a4 + g, inv.y, -oi.y);
    const float t1z = fmaf(a2 - g, inv.z, -oi.z), t2z = fmaf(a5 + g, inv.z, -oi.z);
    const float te = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fmaxf(fminf(t1z, t2z), 0.0f));
    const float tx = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fminf(fmaxf(t1z, t2z), tm));
    return te <= tx;
  };
  auto hit = [&](int ref, float a0, float a1, float a2, float a3, float a4, float a5) {
    if (ref == WALK_EMPTY) return false;
    if (ref >= 0) return slab_hit(a0, a1, a2, a3, a4, a5, 0.0f, tlim);
    return slab_hit(a0, a1, a2, a3, a4, a5, reach, tlim) && slab_hit(a0, a1, a2, a3, a4, a5, 0.0f, INFINITY);
  };
  const bool h0 = hit(rf.x, lx.x, ly.x, lz.x, hx.x, hy.x, hz.x);
  const bool h1 = hit(rf.y, lx.y, ly.y, lz.y, hx.y, hy.y, hz.y);
  const bool h2 = hit(rf.z, lx.z, ly.z, lz.z, hx.z, hy.z, hz.z);
  const bool h3 = hit(rf.w, lx.w, ly.w, lz.w, hx.w, hy.w, hz.w);
  // Enter the first hit child; push the later ones, last first.
  int next = WALK_EMPTY;
  auto take = [&](bool h, int r) {
    if (!h) return;
    if (next != WALK_EMPTY) {
      if (w.sp < RT_STACK4) {
        stack[w.sp++] = next;
      } else {
        atomicOr(err, ERR_STACK_OVERFLOW);
      }
    }
    next = r;
  };
  take(h3, rf.w);
  take(h2, rf.z);
  take(h1, rf.y);
  take(h0, rf.x);
  w.cur = next != WALK_EMPTY ? next : (w.sp > 0 ? stack[--w.sp] : WALK_EMPTY);
}

// Tests the crystals of the lane's oldest queued leaf by their geometry (crystal.rs:140-217) in
// the reference's order, and absorbs each hit inside the step at once (transport.rs:108-138):
// Beer-Lambert, Bernoulli rounding of 5 E p s latent photons, E *= max(1 - 0.9 p, 0.05); the
// n-th absorbing hit of the bounce draws word n % 4 of Philox block n / 4.
__device__ __forceinline__ void leaf_step(const TileDesc& t, const Photon& ph, Bounce& w, uint32_t* err) {
  const uint32_t id = w.lv[0];
#pragma unroll
  for (int j = 0; j + 1 < WALK_LEAVES; ++j) w.lv[j] = w.lv[j + 1];
  w.lv[WALK_LEAVES - 1] = WALK_NONE;
  if (!index_ok(id < t.nnodes, err, SITE_LEAF, id, t.nnodes)) return;
  const uint2 L = __ldg(&t.rleaf[id]);
  if (!index_ok(L.x + L.y <= t.n, err, SITE_LEAF, L.x, L.y)) return;
  const float3 pos = ph.pos, dir = ph.dir;
  const float step = w.step;
  const uint32_t b = ph.b - 1;
  for (uint32_t k = 0; k < L.y; ++k) {
    const uint32_t e = L.x + k;  // element position: the crystal ridx[e]
    const float4 a = __ldg(&t.a[e]), d = __ldg(&t.d[e]);
    // The crystal lies in the ball of radius sqrt(3) m (a cube) or m (the ellipsoid shapes)
    // around its centre; a ball the step's segment misses, with a margin well above FP32
    // rounding, cannot give a hit inside the step, so the geometry test is skipped (the hits
    // and their order are those of testing every crystal).
    {
      const float m = fmaxf(fmaxf(d.x, d.y), d.z);
      const float R = (morph_of(d) == 0 ? 1.7320509f * m : m) * 1.001f + 1e-3f;
      const float wx = a.x - pos.x, wy = a.y - pos.y, wz = a.z - pos.z;
      const float tc = fminf(fmaxf(wx * dir.x + wy * dir.y + wz * dir.z, 0.0f), step);
      const float ex = wx - tc * dir.x, ey = wy - tc * dir.y, ez = wz - tc * dir.z;
      if (ex * ex + ey * ey + ez * ez > R * R) continue;
    }
    const float4 q = __ldg(&t.q[e]);
    float t0, t1;
    if (!fintersect(a, q, d, 1.0f, pos, dir, t0, t1)) continue;
    if (!(t0 < step)) continue;
    const float path = fmaxf(fminf(t1, step) - t0, 0.0f);
    if (!(path > 0.0f)) continue;
    if ((w.nh & 3) == 0) w.r = philox(ph.id, b, w.nh >> 2, TAG_HIT, t.k0, t.k1);
    // 1 - exp(-alpha L) without the cancellation of a short chord (corner hits are common).
    const float p = -expm1f(-t.alpha * path);
    const float expected = w.E * p * a.w * 5.0f;
    const float fl = floorf(expected);
    const uint32_t cnt = static_cast<uint32_t>(fl) + (uf(word(w.r, w.nh & 3)) < expected - fl ? 1u : 0u);
    if (cnt) {
      const uint32_t s = __ldg(&t.ridx[e]);
      if (index_ok(s < t.n, err, SITE_LEAF, s, t.n)) add_counts(t.counts, s, cnt);
    }
    w.E *= fmaxf(1.0f - p * 0.9f, 0.05f);
    ++w.nh;
  }
}

// Ends the bounce whose walk is done (transport.rs:140-185): the move, the film's faces (escape,
// or the anti-halation layer's reflection, optics.rs:150-196), Henyey-Greenstein scattering with
// albedo and Russian roulette.  Returns whether the packet is still alive.
__device__ __forceinline__ bool bounce_end(const TileDesc& t, Photon& ph, const Bounce& w) {
  const float PI2 = 6.283185307179586f;
  const uint32_t b = ph.b - 1;
  const P4 rb = philox(ph.id, b, 0, TAG_BOUNCE, t.k0, t.k1);
  const float3 pos = ph.pos, dir = ph.dir;
  const float step = w.step;
  float E = w.E;
  const float3 np = make_float3(pos.x + dir.x * step, pos.y + dir.y * step, pos.z + dir.z * step);
  if (np.x < 0.0f || np.x >= t.W || np.y < 0.0f || np.y >= t.H) return false;
  if (np.z <= 0.0f) return false;
  if (np.z >= t.D) {
    ph.pos = make_float3(np.x, np.y, t.D - 0.001f);
    const P4 ra = philox(ph.id, b, 0, TAG_AH, t.k0, t.k1);
    E *= t.eff_r;
    if (E < 1e-4f) {
      if (uf(ra.x) < 0.1f) E /= 0.1f; else return false;
    }
    float3 d2;
    if (uf(ra.y) < 0.4f) {
      const float u1 = uf(ra.z), u2 = uf(ra.w);
      const float rr = sqrtf(u1);
      float s2, c2;
      sincosf(PI2 * u2, &s2, &c2);
      d2 = make_float3(rr * c2, rr * s2, -sqrtf(fmaxf(1.0f - u1, 0.0f)));
    } else {
      d2 = make_float3(dir.x, dir.y, -fabsf(dir.z));
    }
    const float n = rsqrtf(d2.x * d2.x + d2.y * d2.y + d2.z * d2.z);
    ph.dir = make_float3(d2.x * n, d2.y * n, d2.z * n);
    ph.E = E;
    return true;
  }
  ph.pos = np;
  float cth;
  if (fabsf(t.g) < 1e-4f) {
    cth = 2.0f * uf(rb.y) - 1.0f;
  } else {
    const float term = (1.0f - t.g * t.g) / (1.0f - t.g + 2.0f * t.g * uf(rb.y));
    cth = (1.0f + t.g * t.g - term * term) / (2.0f * t.g);
  }
  cth = fminf(fmaxf(cth, -1.0f), 1.0f);
  const float sth = sqrtf(fmaxf(1.0f - cth * cth, 0.0f));
  float sph, cph;
  sincosf(PI2 * uf(rb.z), &sph, &cph);
  float3 u = fabsf(dir.x) > 0.1f ? make_float3(dir.z, 0.0f, -dir.x) : make_float3(0.0f, -dir.z, dir.y);
  {
    const float n = rsqrtf(u.x * u.x + u.y * u.y + u.z * u.z);
    u = make_float3(u.x * n, u.y * n, u.z * n);
  }
  const float3 v = make_float3(dir.y * u.z - dir.z * u.y, dir.z * u.x - dir.x * u.z, dir.x * u.y - dir.y * u.x);
  const float3 nd = make_float3(u.x * sth * cph + v.x * sth * sph + dir.x * cth,
                                u.y * sth * cph + v.y * sth * sph + dir.y * cth,
                                u.z * sth * cph + v.z * sth * sph + dir.z * cth);
  const float n = rsqrtf(nd.x * nd.x + nd.y * nd.y + nd.z * nd.z);
  ph.dir = make_float3(nd.x * n, nd.y * n, nd.z * n);
  E *= t.albedo;
  if (E < 1e-3f) {
    if (uf(rb.w) < 0.1f) E /= 0.1f; else return false;
  }
  ph.E = E;
  return true;
}

}  // namespace fg
