// Device code of the photon transport: tile descriptors, the LBVH walk and the per-photon
// bounce loop (transport.rs:101-185, optics.rs:100-196).
#pragma once
#include "fg_device.cuh"

namespace fg {

constexpr int HMAX = 48;  // hits kept per segment (a 21 um segment meets ~10 crystals)

// Everything one tile's transport needs, 16-byte aligned for vector loads.
struct __align__(16) TileDesc {
  const float4* a;
  const float4* q;
  const float4* d;
  const Node* nodes;
  const uint32_t* s2id;
  uint32_t* counts;
  const float* tile;
  unsigned long long photon_base;
  uint32_t n, tw, th, P;
  uint32_t stride;  // exposure row stride (floats); tiles may be windows of one image
  float W, H, D;
  uint32_t k0, k1;
  float mu_t, albedo, g, r0, eff_r, theta_max, alpha;
  uint32_t max_bounces;
};

// Stack walk of the LBVH: fn(s) is called for every crystal whose padded leaf box the ray
// enters before tlim.  Both child boxes come with the parent, so each step is one node load.
template <class F>
__device__ __forceinline__ void walk_lbvh(const Node* __restrict__ nodes, float3 o, float3 inv,
                                          float tlim, uint32_t* err, F&& fn) {
  int stack[64];
  int sp = 0;
  int cur = 0;
  for (;;) {
    const float4 na = __ldg(&nodes[cur].a);
    const float4 nb = __ldg(&nodes[cur].b);
    const float4 nc = __ldg(&nodes[cur].c);
    const int4 nd = __ldg(&nodes[cur].d);
    float te, tx;
    slab(o, inv, na.x, na.y, na.z, na.w, nb.x, nb.y, te, tx);
    bool hl = tx >= te && tx >= 0.0f && te <= tlim;
    slab(o, inv, nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, te, tx);
    bool hr = tx >= te && tx >= 0.0f && te <= tlim && nd.y != INT32_MIN;
    if (hl && nd.x < 0) {
      fn(static_cast<uint32_t>(~nd.x));
      hl = false;
    }
    if (hr && nd.y < 0) {
      fn(static_cast<uint32_t>(~nd.y));
      hr = false;
    }
    if (hl && hr) {
      if (sp < 64) {
        stack[sp++] = nd.y;
      } else {
        atomicOr(err, ERR_STACK_OVERFLOW);
      }
      cur = nd.x;
    } else if (hl) {
      cur = nd.x;
    } else if (hr) {
      cur = nd.y;
    } else {
      if (sp == 0) break;
      cur = stack[--sp];
    }
  }
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

struct HitF {
  float t0, t1;
  uint32_t id, s;
};

// Adds n latent photons to crystal s, one atomic per distinct crystal among the active lanes.
__device__ __forceinline__ void add_counts(uint32_t* counts, uint32_t s, uint32_t n) {
  const unsigned act = __activemask();
  const unsigned grp = __match_any_sync(act, s);
  const int leader = __ffs(grp) - 1;
  uint32_t sum = 0;
  for (unsigned m = grp; m; m &= m - 1) sum += __shfl_sync(grp, n, __ffs(m) - 1);
  if ((threadIdx.x & 31) == leader && sum) atomicAdd(&counts[s], sum);
}

// One photon packet from emission to death (transport.rs:72-185).  Returns its absorbing hits.
static __device__ __noinline__ uint32_t trace_photon(const TileDesc& t, uint32_t id, uint32_t* err) {
  const float PI2 = 6.283185307179586f;
  const P4 e0 = philox(id, 0, 0, TAG_EMIT, t.k0, t.k1);
  const float x = uf(e0.x) * t.W;
  const float y = uf(e0.y) * t.H;
  // Nearest-pixel exposure closure (image_pipeline.rs:949-958).
  const float uu = fminf(fmaxf(x / t.W, 0.0f), 1.0f), vv = fminf(fmaxf(y / t.H, 0.0f), 1.0f);
  const uint32_t px = min(static_cast<uint32_t>(roundf(uu * (float)(t.tw - 1))), t.tw - 1);
  const uint32_t py = min(static_cast<uint32_t>(roundf(vv * (float)(t.th - 1))), t.th - 1);
  float E = fmaxf(__ldg(&t.tile[static_cast<size_t>(py) * t.stride + px]), 0.0f);
  if (!(E > 0.0f)) return 0;
  const float theta = uf(e0.z) * t.theta_max;
  const float phi = uf(e0.w) * PI2;
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(phi, &sp, &cp);
  float3 dir = make_float3(st * cp, st * sp, ct);
  {
    const float n = rsqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
    dir = make_float3(dir.x * n, dir.y * n, dir.z * n);
  }
  // Schlick reflectance at the air-gelatin interface (optics.rs:147-154).
  const float c = fminf(fabsf(dir.z), 1.0f), m = 1.0f - c, m2 = m * m;
  const float R = t.r0 + (1.0f - t.r0) * (m2 * m2 * m);
  const P4 e1 = philox(id, 0, 1, TAG_EMIT, t.k0, t.k1);
  if (uf(e1.x) < R) return 0;
  float3 pos = make_float3(x, y, 0.001f);
  uint32_t nhits_total = 0;
  HitF hits[HMAX];
  for (uint32_t b = 0; b < t.max_bounces; ++b) {
    const P4 rb = philox(id, b, 0, TAG_BOUNCE, t.k0, t.k1);
    const float fp = t.mu_t > 0.0f ? -__logf(fmaxf(1.0f - uf(rb.x), 1.17549435e-38f)) / t.mu_t : 1e6f;
    const float step = fminf(fp, t.D * 1.5f);
    const float3 inv = make_float3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    int nh = 0;
    if (t.n > 0) {
      walk_lbvh(t.nodes, pos, inv, step * 1.00001f + 1e-3f, err, [&](uint32_t s) {
        const float4 a = __ldg(&t.a[s]), q = __ldg(&t.q[s]), d = __ldg(&t.d[s]);
        float t0, t1;
        if (!fcanonical_hit(a, q, d, 1.0f, pos, dir, inv, t0, t1)) return;
        if (!(t0 < step)) return;
        if (!(fmaxf(fminf(t1, step) - t0, 0.0f) > 0.0f)) return;
        const uint32_t cid = t.s2id ? __ldg(&t.s2id[s]) : s;
        if (nh == HMAX) { atomicOr(err, ERR_HIT_OVERFLOW); return; }
        int j = nh++;
        while (j > 0 && (hits[j - 1].t0 > t0 || (hits[j - 1].t0 == t0 && hits[j - 1].id > cid))) {
          hits[j] = hits[j - 1];
          --j;
        }
        hits[j] = HitF{t0, t1, cid, s};
      });
    }
    P4 r{};
    for (int h = 0; h < nh; ++h) {
      if ((h & 3) == 0) r = philox(id, b, static_cast<uint32_t>(h) >> 2, TAG_HIT, t.k0, t.k1);
      const float path = fmaxf(fminf(hits[h].t1, step) - hits[h].t0, 0.0f);
      const float p = 1.0f - __expf(-t.alpha * path);
      const float expected = E * p * __ldg(&t.a[hits[h].s].w) * 5.0f;
      const float fl = floorf(expected);
      const float frac = expected - fl;
      const uint32_t cnt = static_cast<uint32_t>(fl) + (uf(word(r, h & 3)) < frac ? 1u : 0u);
      if (cnt) add_counts(t.counts, hits[h].s, cnt);
      E *= fmaxf(1.0f - p * 0.9f, 0.05f);
    }
    nhits_total += nh;
    const float3 np = make_float3(pos.x + dir.x * step, pos.y + dir.y * step, pos.z + dir.z * step);
    if (np.x < 0.0f || np.x >= t.W || np.y < 0.0f || np.y >= t.H) break;
    if (np.z <= 0.0f) break;
    if (np.z >= t.D) {
      // Anti-halation backing (optics.rs:160-196).
      pos = make_float3(np.x, np.y, t.D - 0.001f);
      const P4 ra = philox(id, b, 0, TAG_AH, t.k0, t.k1);
      E *= t.eff_r;
      if (E < 1e-4f) {
        if (uf(ra.x) < 0.1f) E /= 0.1f; else break;
      }
      if (uf(ra.y) < 0.4f) {
        const float u1 = uf(ra.z), u2 = uf(ra.w);
        const float r = sqrtf(u1);
        float s2, c2;
        sincosf(PI2 * u2, &s2, &c2);
        dir = make_float3(r * c2, r * s2, -sqrtf(fmaxf(1.0f - u1, 0.0f)));
      } else {
        dir.z = -fabsf(dir.z);
      }
      const float n = rsqrtf(dir.x * dir.x + dir.y * dir.y + dir.z * dir.z);
      dir = make_float3(dir.x * n, dir.y * n, dir.z * n);
      continue;
    }
    pos = np;
    // Henyey-Greenstein scattering (optics.rs:113-143).
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
    float3 u;
    if (fabsf(dir.x) > 0.1f) {
      u = make_float3(dir.z, 0.0f, -dir.x);  // (0,1,0) x w
    } else {
      u = make_float3(0.0f, -dir.z, dir.y);  // (1,0,0) x w
    }
    {
      const float n = rsqrtf(u.x * u.x + u.y * u.y + u.z * u.z);
      u = make_float3(u.x * n, u.y * n, u.z * n);
    }
    const float3 v = make_float3(dir.y * u.z - dir.z * u.y, dir.z * u.x - dir.x * u.z, dir.x * u.y - dir.y * u.x);
    float3 nd = make_float3(u.x * sth * cph + v.x * sth * sph + dir.x * cth,
                            u.y * sth * cph + v.y * sth * sph + dir.y * cth,
                            u.z * sth * cph + v.z * sth * sph + dir.z * cth);
    const float n = rsqrtf(nd.x * nd.x + nd.y * nd.y + nd.z * nd.z);
    dir = make_float3(nd.x * n, nd.y * n, nd.z * n);
    E *= t.albedo;
    if (E < 1e-3f) {
      if (uf(rb.w) < 0.1f) E /= 0.1f; else break;
    }
  }
  return nhits_total;
}

}  // namespace fg
