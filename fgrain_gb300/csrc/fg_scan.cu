// Transmittance scan kernels: binning of developed crystals and the binned scan itself.
#include "fg_internal.h"
#include "fg_scan.cuh"

namespace fg {

// Bin range [lo, hi] (um, padded by 1e-3) in one axis.
__device__ __forceinline__ void bin_span(double lo, double hi, float binw, uint32_t nb, uint32_t& b0, uint32_t& b1) {
  const float l = (static_cast<float>(lo) - 1e-3f) / binw, h = (static_cast<float>(hi) + 1e-3f) / binw;
  const float fl = fminf(fmaxf(floorf(l), 0.0f), (float)(nb - 1));
  const float fh = fminf(fmaxf(floorf(h), 0.0f), (float)(nb - 1));
  b0 = static_cast<uint32_t>(fl);
  b1 = static_cast<uint32_t>(fh);
}

// Bins of developed crystal s: those its leaf box overlaps (a ray outside the leaf box misses s).
__device__ __forceinline__ void leaf_bins(const ScanTile& t, uint32_t s, uint32_t& x0, uint32_t& x1, uint32_t& y0,
                                          uint32_t& y1) {
  const double* b = t.lbox64 + 6ull * t.leafof[s];
  bin_span(b[0], b[3], (float)(t.bin_px * t.pw), t.nbx, x0, x1);
  bin_span(b[1], b[4], (float)(t.bin_px * t.ph), t.nby, y0, y1);
}

__global__ void k_bin_count(ScanTile t, uint32_t* cnt) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= t.n || !t.developed[s]) return;
  uint32_t x0, x1, y0, y1;
  leaf_bins(t, s, x0, x1, y0, y1);
  for (uint32_t by = y0; by <= y1; ++by)
    for (uint32_t bx = x0; bx <= x1; ++bx) atomicAdd(&cnt[by * t.nbx + bx], 1u);
}

__global__ void k_bin_fill(ScanTile t, const uint32_t* off, uint32_t* cursor, uint32_t* items) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= t.n || !t.developed[s]) return;
  uint32_t x0, x1, y0, y1;
  leaf_bins(t, s, x0, x1, y0, y1);
  for (uint32_t by = y0; by <= y1; ++by)
    for (uint32_t bx = x0; bx <= x1; ++bx) {
      const uint32_t b = by * t.nbx + bx;
      items[off[b] + atomicAdd(&cursor[b], 1u)] = s;
    }
}

// Error-free transformations on floats (Knuth's two-sum, FMA two-product).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
__device__ __forceinline__ void split64(double v, float& hi, float& lo) {
  hi = static_cast<float>(v);
  lo = static_cast<float>(v - static_cast<double>(hi));
}
// A float widened to double by moving its bits (integer pipes); zero and subnormals (T below
// 2^-126, rare) take the conversion instruction.
__device__ __forceinline__ double f2d_exact(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return static_cast<double>(f);
  const unsigned long long d = (static_cast<unsigned long long>(b & 0x80000000u) << 32) |
                               (static_cast<unsigned long long>(e + (1023u - 127u)) << 52) |
                               (static_cast<unsigned long long>(b & 0x7fffffu) << 29);
  return __longlong_as_double(static_cast<long long>(d));
}

// (ah + al) - (bh + bl) as a float pair, to about 2^-48 of the operands.
__device__ __forceinline__ void pair_sub(float ah, float al, float bh, float bl, float& h, float& l) {
  float s, e;
  two_sum(ah, -bh, s, e);
  two_sum(s, e + (al - bl), h, l);
}

// Fixed-point chord sums (units of 2^-40 um) without 64-bit integer / float conversions, which
// run on GB300's narrow FP64 pipe.  fix40(v) equals __float2ll_rn(v * 2^40) for 0 <= v < 2^15:
// below 2^31 the 32-bit conversion rounds the same way; above, v * 2^40 is an integer (its ulp is
// at least 2^8) split exactly into hi * 2^24 + lo.
__device__ __forceinline__ long long fix40(float v) {
  const float w = v * 1099511627776.0f;
  if (w < 2147483648.0f) return static_cast<long long>(__float2int_rn(w));
  const float hf = truncf(w * 0x1p-24f);
  const float lf = fmaf(-hf, 16777216.0f, w);  // exact: the low 24 bits of an integer
  return (static_cast<long long>(__float2int_rz(hf)) << 24) + __float2int_rz(lf);
}
// u rounded to the nearest float (ties to even), as __ll2float_rn does, in integer arithmetic.
__device__ __forceinline__ float u64_to_float_rn(unsigned long long u) {
  if (u < (1ull << 24)) return static_cast<float>(static_cast<uint32_t>(u));
  const int sh = 63 - __clzll(static_cast<long long>(u)) - 23;  // >= 1
  unsigned long long m = u >> sh;                                // 24 bits
  const unsigned long long rem = u & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
  if (rem > half || (rem == half && (m & 1ull))) ++m;            // m <= 2^24: exact as a float
  return static_cast<float>(static_cast<uint32_t>(m)) * __int_as_float((127 + sh) << 23);
}

// Crystal kinds in shared memory.
enum : int { K_CUBE = 0, K_CUBE_DF = 1, K_ELLIPSOID = 2, K_FP64 = 3 };

// Shared-memory image of a staged crystal (index c of the current chunk).  Coordinates are
// relative to the bin corner and carried as float pairs (hi + lo) so that ray-minus-crystal
// offsets are accurate to ~1e-8 um.
struct ScanSmem {
  float cxh[SCAN_CH], cxl[SCAN_CH], cyh[SCAN_CH], cyl[SCAN_CH];
  // Leaf box x / y extent relative to the corner, float pairs: x0, x1, y0, y1.
  float lbh[4][SCAN_CH], lbl[4][SCAN_CH];
  float m[SCAN_CH], delta[SCAN_CH], err[SCAN_CH], sig[SCAN_CH];
  float g[21][SCAN_CH];
  int s[SCAN_CH];
  int kind[SCAN_CH];
  double T[SCAN_THREADS];
};

constexpr float EPS32 = 5.9604645e-8f;  // 2^-24

// Stages crystal s for vertical rays relative to the bin corner (bx0, by0).  Everything is
// derived in FP64 once per crystal and CTA, then rounded:
//   cubes:      rows 0 and 1 of R as float pairs, 1 / (-R_2i), half-sizes as float pairs;
//   ellipsoids: R_0i / D_i, R_1i / D_i, e_i = -R_2i / D_i, A = |e|^2, 1 / A.
// Cubes whose faces are nearly parallel to the ray (|1/R_2i| > 15) evaluate their local origin in
// float-pair arithmetic; cubes with an exactly parallel face decide in FP64.
__device__ __forceinline__ void prep_crystal(const ScanTile& t, uint32_t s, ScanPrep& P) {
  const Crystal64 k = load64_parts(t, s);
  const double e64 = t.exp64[s];
  const double mdim = fmax(fmax(k.dims.x, k.dims.y), k.dims.z);
  const double m64 = __dmul_rn(mdim, e64);
  const float m = static_cast<float>(m64);
  split64(k.pos.x, P.ch[0], P.cl[0]);
  split64(k.pos.y, P.ch[1], P.cl[1]);
  const double* lb = t.lbox64 + 6ull * t.leafof[s];
  split64(lb[0], P.ch[2], P.cl[2]);
  split64(lb[3], P.ch[3], P.cl[3]);
  split64(lb[1], P.ch[4], P.cl[4]);
  split64(lb[4], P.ch[5], P.cl[5]);
  P.m = m;
  P.delta = static_cast<float>(t.z0 - k.pos.z);
  P.sig = t.sigma_c ? t.sigma_c[s] : t.sigma;
  const double x = k.q[0], y = k.q[1], z = k.q[2], w = k.q[3];
  // world = R local + p, so local_i = R_0i dx + R_1i dy + R_2i dz: rows 0..2 of R.
  const double R0[3] = {1.0 - 2.0 * (y * y + z * z), 2.0 * (x * y - z * w), 2.0 * (x * z + y * w)};
  const double R1[3] = {2.0 * (x * y + z * w), 1.0 - 2.0 * (x * x + z * z), 2.0 * (y * z - x * w)};
  const double R2[3] = {2.0 * (x * z - y * w), 2.0 * (y * z + x * w), 1.0 - 2.0 * (x * x + y * y)};
  const double D[3] = {k.dims.x * e64, k.dims.y * e64, k.dims.z * e64};
#pragma unroll
  for (int i = 0; i < 21; ++i) P.g[i] = 0.0f;
  if (k.morph == 0) {
    float invmax = 0.0f;
    const float Dmax = static_cast<float>(fmax(fmax(D[0], D[1]), D[2]));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      split64(R0[i], P.g[i], P.g[3 + i]);
      split64(R1[i], P.g[6 + i], P.g[9 + i]);
      const float inv = static_cast<float>(1.0 / (-R2[i]));
      P.g[12 + i] = inv;
      split64(D[i], P.g[15 + i], P.g[18 + i]);
      invmax = fmaxf(invmax, fabsf(inv));
    }
    if (!(invmax < 1e30f)) {
      P.kind = K_FP64;
      P.err = INFINITY;
    } else if (invmax > 15.0f) {
      P.kind = K_CUBE_DF;
      P.err = 0.0f;  // bounds are formed per ray from the t values
    } else {
      P.kind = K_CUBE;
      // A cube lies within sqrt(3) m of its centre, so rays that can hit it are within mr of the
      // centre in x and y.  |d local| <= 4e-7 mr + 1e-7 (rounded rows, offsets); |d D| <= eps D;
      // each t = (+-D - lo) * inv carries (d lo + d D) |inv| + 2 eps |t|, with |t| <= (D + 2 mr)
      // invmax.
      const float mr = 1.7320509f * m;
      P.err = 4.0f * ((4e-7f * mr + 1e-7f + EPS32 * Dmax) * invmax + 2.0f * EPS32 * (Dmax + 2.0f * mr) * invmax);
    }
  } else {
    P.kind = K_ELLIPSOID;
    double A = 0.0;
    const double Dmin = fmin(fmin(D[0], D[1]), D[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      P.g[i] = static_cast<float>(R0[i] / D[i]);
      P.g[3 + i] = static_cast<float>(R1[i] / D[i]);
      const double ei = -R2[i] / D[i];
      P.g[6 + i] = static_cast<float>(ei);
      A += ei * ei;
    }
    P.g[9] = static_cast<float>(A);
    P.g[10] = static_cast<float>(1.0 / A);
    // h = 1 - |P_perp|^2; P (|P| <= sqrt(2) m / Dmin) and P_perp = P + tc e carry ~8 eps |P|
    // each, so |d h| <= 2 |P_perp| 8 eps sqrt(3) Pmax + 4 eps; four times that as the bound.
    const float Pmax = static_cast<float>(1.4142135623730951 * m64 / Dmin);
    P.err = 4.0f * (2.0f * 1.05f * 8.0f * EPS32 * 1.7320508f * Pmax + 4.0f * EPS32) + 1e-9f;
  }
}

// Stages crystal s for the bin whose 16-px-square corner is (bxh + bxl, byh + byl): the
// bin-independent terms (from t.prep, or derived here), and the centre and leaf box relative to
// the corner as float pairs (float arithmetic only).
__device__ __forceinline__ void stage_crystal(const ScanTile& t, ScanSmem& sm, int c, uint32_t s, float bxh,
                                              float bxl, float byh, float byl) {
  ScanPrep P;
  if (t.prep) {
    P = t.prep[s];
  } else {
    prep_crystal(t, s, P);
  }
  pair_sub(P.ch[0], P.cl[0], bxh, bxl, sm.cxh[c], sm.cxl[c]);
  pair_sub(P.ch[1], P.cl[1], byh, byl, sm.cyh[c], sm.cyl[c]);
  pair_sub(P.ch[2], P.cl[2], bxh, bxl, sm.lbh[0][c], sm.lbl[0][c]);
  pair_sub(P.ch[3], P.cl[3], bxh, bxl, sm.lbh[1][c], sm.lbl[1][c]);
  pair_sub(P.ch[4], P.cl[4], byh, byl, sm.lbh[2][c], sm.lbl[2][c]);
  pair_sub(P.ch[5], P.cl[5], byh, byl, sm.lbh[3][c], sm.lbl[3][c]);
  sm.m[c] = P.m;
  sm.delta[c] = P.delta;
  sm.err[c] = P.err;
  sm.sig[c] = P.sig;
  sm.kind[c] = P.kind;
  sm.s[c] = static_cast<int>(s);
#pragma unroll
  for (int i = 0; i < 21; ++i) sm.g[i][c] = P.g[i];
}

// Staging terms of every developed crystal of every tile, once per crystal (k_scan reads them).
__global__ void k_scan_prep(const ScanTile* __restrict__ tiles, int ntiles, unsigned long long nslots,
                            ScanPrep* __restrict__ prep) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= nslots) return;
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].slot_base <= g) lo = mid; else hi = mid - 1;
  }
  const ScanTile& t = tiles[lo];
  const unsigned long long s = g - t.slot_base;
  if (s >= t.n || !t.developed[s]) return;
  ScanPrep P;
  prep_crystal(t, static_cast<uint32_t>(s), P);
  prep[g] = P;
}

// k_scan_prep over a list of the developed crystals' slots (*nlist of them, at most cap): one
// thread per listed crystal, so the FP64 derivation runs with every lane busy.
__global__ void k_scan_prep_list(const ScanTile* __restrict__ tiles, int ntiles, const uint32_t* __restrict__ list,
                                 const uint32_t* __restrict__ nlist, unsigned long long cap,
                                 ScanPrep* __restrict__ prep) {
  const unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (i >= cap || i >= *nlist) return;
  const unsigned long long g = list[i];
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].slot_base <= g) lo = mid; else hi = mid - 1;
  }
  const ScanTile& t = tiles[lo];
  const unsigned long long s = g - t.slot_base;
  if (s >= t.n || !t.developed[s]) return;
  ScanPrep P;
  prep_crystal(t, static_cast<uint32_t>(s), P);
  prep[g] = P;
}

void launch_scan_prep_list(const ScanTile* tiles, int ntiles, const uint32_t* list, const uint32_t* nlist,
                           unsigned long long cap, ScanPrep* prep, cudaStream_t st) {
  if (cap == 0) return;
  k_scan_prep_list<<<grid_for(cap, 128), 128, 0, st>>>(tiles, ntiles, list, nlist, cap, prep);
  FG_CUDA(cudaGetLastError());
}

void launch_scan_prep(const ScanTile* tiles, int ntiles, unsigned long long nslots, ScanPrep* prep,
                      cudaStream_t st) {
  if (nslots == 0) return;
  k_scan_prep<<<grid_for(nslots, 128), 128, 0, st>>>(tiles, ntiles, nslots, prep);
  FG_CUDA(cudaGetLastError());
}

// Decision and chord of one scanner ray against staged crystal c.  The ray's origin is a float pair
// relative to the bin's 16-px corner; a pair whose decision falls inside its error bound is
// decided with the reference's FP64 expressions (counted in nfb).
__device__ __forceinline__ bool scan_pair(const ScanTile& t, const ScanSmem& sm, uint32_t c, float oxh, float oxl,
                                          float oyh, float oyl, uint32_t px, uint32_t py, uint32_t sx, uint32_t sy,
                                          float& chord, uint32_t& nfb) {
  const float m = sm.m[c], delta = sm.delta[c];
  const int kind = sm.kind[c];
  // Geometry reach: a cube lies within sqrt(3) m of its centre, an ellipsoid within its own box.
  const float reach = (kind == K_ELLIPSOID ? m : 1.7320509f * m) * 1.00001f + 1e-9f;
  {
    // Quick rejection on the high words alone: they differ from the float pairs by a few units in
    // the last place, far inside the slack, so a pair rejected here fails the exact test below.
    const float cxh = sm.cxh[c], cyh = sm.cyh[c];
    const float slack = 1e-4f + 4.8e-7f * (fabsf(oxh) + fabsf(cxh) + fabsf(oyh) + fabsf(cyh));
    if (fabsf(oxh - cxh) > reach + slack || fabsf(oyh - cyh) > reach + slack) return false;
  }
  // Ray minus crystal centre, x and y, as float pairs.
  float dh, dl, dx, dxl, dy, dyl;
  two_sum(oxh, -sm.cxh[c], dh, dl);
  fast_two_sum(dh, dl + (oxl - sm.cxl[c]), dx, dxl);
  two_sum(oyh, -sm.cyh[c], dh, dl);
  fast_two_sum(dh, dl + (oyl - sm.cyl[c]), dy, dyl);
  if (fabsf(dx) > reach || fabsf(dy) > reach) return false;
  // The leaf box (strict containment in x and y; the origin lies above every box in z): margins
  // of float-pair differences, exact to ~1e-12 um.
  float lm = INFINITY;
  {
    float h, l;
    two_sum(oxh, -sm.lbh[0][c], h, l);
    lm = fminf(lm, h + (l + (oxl - sm.lbl[0][c])));
    two_sum(sm.lbh[1][c], -oxh, h, l);
    lm = fminf(lm, h + (l + (sm.lbl[1][c] - oxl)));
    two_sum(oyh, -sm.lbh[2][c], h, l);
    lm = fminf(lm, h + (l + (oyl - sm.lbl[2][c])));
    two_sum(sm.lbh[3][c], -oyh, h, l);
    lm = fminf(lm, h + (l + (sm.lbl[3][c] - oyl)));
  }
  const float EBL = 1e-9f;
  if (lm < -EBL) return false;
  bool amb = lm <= EBL || kind == K_FP64;
  bool hit = false;
  chord = 0.0f;
  if (!amb) {
    if (kind != K_ELLIPSOID) {
      float tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float inv = sm.g[12 + i][c], Dh = sm.g[15 + i][c];
        float a1, a2;
        if (kind == K_CUBE) {
          const float lo_i = fmaf(sm.g[i][c], dx, sm.g[6 + i][c] * dy);
          a1 = -Dh - lo_i;
          a2 = Dh - lo_i;
        } else {
          // Local origin as a float pair, then the two face offsets exactly rounded.
          const float R0h = sm.g[i][c], R0l = sm.g[3 + i][c], R1h = sm.g[6 + i][c], R1l = sm.g[9 + i][c];
          const float Dl = sm.g[18 + i][c];
          float p0, e0, p1, e1, sh, sl;
          two_prod(R0h, dx, p0, e0);
          two_prod(R1h, dy, p1, e1);
          two_sum(p0, p1, sh, sl);
          sl += (e0 + e1) + ((R0h * dxl + R1h * dyl) + (R0l * dx + R1l * dy));
          float v, wv;
          two_sum(-Dh, -sh, v, wv);
          a1 = v + ((wv - Dl) - sl);
          two_sum(Dh, -sh, v, wv);
          a2 = v + ((wv + Dl) - sl);
        }
        const float t1 = a1 * inv, t2 = a2 * inv;
        tmin = fmaxf(tmin, fminf(t1, t2));
        tmax = fminf(tmax, fmaxf(t1, t2));
      }
      const float E = kind == K_CUBE ? sm.err[c] : 4.0f * 3.0f * EPS32 * (fabsf(tmin) + fabsf(tmax)) + 1e-9f;
      const float m1 = tmax - tmin, m2 = tmax + delta;
      const float E2 = E + 4.0f * 3.0f * EPS32 * fabsf(delta) + 2e-6f;
      if (m1 > 2.0f * E && m2 > E2) {
        hit = true;
        chord = tmax - fmaxf(tmin, -delta);
      } else if (!(m1 < -2.0f * E || m2 < -E2)) {
        amb = true;
      }
    } else {
      float P[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) P[i] = fmaf(sm.g[i][c], dx, sm.g[3 + i][c] * dy);
      const float e0 = sm.g[6][c], e1 = sm.g[7][c], e2 = sm.g[8][c];
      const float iA = sm.g[10][c];
      // Closest approach along the ray (t' = tc) and the offset there: h = 1 - |P_perp|^2
      // has the sign of the reference's discriminant.
      const float tc = -(P[0] * e0 + P[1] * e1 + P[2] * e2) * iA;
      const float q0 = fmaf(tc, e0, P[0]), q1 = fmaf(tc, e1, P[1]), q2 = fmaf(tc, e2, P[2]);
      const float hh = 1.0f - (q0 * q0 + q1 * q1 + q2 * q2);
      const float E = sm.err[c];
      if (hh > E) {
        const float sq = sqrtf(hh * iA);
        const float t0 = tc - sq, t1 = tc + sq;
        const float E2 = 4.0f * 3.0f * EPS32 * (fabsf(t1) + fabsf(delta)) + 2e-6f;
        if (t1 + delta > E2) {
          hit = true;
          chord = t1 - fmaxf(t0, -delta);
        } else {
          amb = true;
        }
      } else if (!(hh < -E)) {
        amb = true;
      }
    }
  }
  if (amb) {
    ++nfb;
    double ox64, oy64;
    scan_origin64(t, px, py, sx, sy, ox64, oy64);
    bool h64;
    const double c64 = scan_chord64(t, static_cast<uint32_t>(sm.s[c]), ox64, oy64, h64);
    hit = h64;
    chord = static_cast<float>(c64);
  }
  return hit;
}

// One thread's scanner ray in a bin: pixel, stratum and the ray origin relative to the corner of
// the 16-pixel square holding the bin (float pairs), shared by the forward scan and its adjoint.
struct ScanRay {
  uint32_t px, py, sx, sy, st;
  bool active;
  float bxh, bxl, byh, byl;  // corner of the 16-pixel square holding the bin (um, float pairs)
  float oxh, oxl, oyh, oyl;
};

__device__ __forceinline__ ScanRay scan_ray(const ScanTile& t, uint32_t bin, uint32_t tid) {
  ScanRay R;
  const uint32_t bx = bin % t.nbx, by = bin / t.nbx;
  const uint32_t a = t.spp;
  const uint32_t pix = tid / a, st = tid % a;
  const uint32_t lx = pix % t.bin_px, ly = pix / t.bin_px;
  const uint32_t px = bx * t.bin_px + lx, py = by * t.bin_px + ly;
  const bool active = pix < t.bin_px * t.bin_px && px < t.w && py < t.h;
  const uint32_t sx = st % t.g, sy = st / t.g;
  // Coordinates are taken relative to the corner of the 16-pixel square holding this bin, not to
  // the bin itself, so that every bin edge rounds identically and results do not depend on the
  // launch shape.
  const uint32_t ox_px = (bx * t.bin_px) & ~15u, oy_px = (by * t.bin_px) & ~15u;
  {
    // The corner as a whole number of jitter units, (ox_px g 2^24) (pw / (g 2^24)), in float pairs:
    // the ray offsets below are counted in the same units, so the two agree to about 2^-48.
    const float fx = static_cast<float>(ox_px * t.g) * 16777216.0f, fy = static_cast<float>(oy_px * t.g) * 16777216.0f;
    float p, e;
    two_prod(fx, t.jxh, p, e);
    fast_two_sum(p, fmaf(fx, t.jxl, e), R.bxh, R.bxl);
    two_prod(fy, t.jyh, p, e);
    fast_two_sum(p, fmaf(fy, t.jyl, e), R.byh, R.byl);
  }
  const uint32_t rlx = px - ox_px, rly = py - oy_px;  // < 16 + bin_px
  // Ray position relative to that corner as a float pair.  The offset in units of the 24-bit
  // jitter is an exact integer X = (l g + s) 2^24 + u, so x = X * pw / (g 2^24).
  float oxh = 0.0f, oxl = 0.0f, oyh = 0.0f, oyl = 0.0f;
  if (active) {
    const uint64_t ps = t.seed + static_cast<uint64_t>(px) * 0x9E3779B97F4A7C15ull +
                        static_cast<uint64_t>(py) * 0xC6A4A7935BD1E995ull;
    const P4 r = philox(sy * t.g + sx, 0, 0, TAG_SCAN, static_cast<uint32_t>(ps), static_cast<uint32_t>(ps >> 32));
    const float cxh = t.jxh, cxl = t.jxl, cyh = t.jyh, cyl = t.jyl;
    const uint32_t X = ((rlx * t.g + sx) << 24) + (r.x >> 8);
    const uint32_t Y = ((rly * t.g + sy) << 24) + (r.y >> 8);
    // X, Y < 2^31 as a float pair: Xh rounded, Xl = X - Xh exact (32-bit conversions only; the
    // 64-bit ones run on the FP64 pipe).
    const float Xh = __uint2float_rn(X), Yh = __uint2float_rn(Y);
    const float Xl = __int2float_rn(static_cast<int>(X - __float2uint_rn(Xh)));
    const float Yl = __int2float_rn(static_cast<int>(Y - __float2uint_rn(Yh)));
    float p, e;
    two_prod(Xh, cxh, p, e);
    fast_two_sum(p, e + (Xh * cxl + Xl * cxh), oxh, oxl);
    two_prod(Yh, cyh, p, e);
    fast_two_sum(p, e + (Yh * cyl + Yl * cyh), oyh, oyl);
  }
  R.px = px;
  R.py = py;
  R.sx = sx;
  R.sy = sy;
  R.st = st;
  R.active = active;
  R.oxh = oxh;
  R.oxl = oxl;
  R.oyh = oyh;
  R.oyl = oyl;
  return R;
}

// Tile of global bin gb (last tile whose first bin <= gb).
__device__ __forceinline__ int scan_tile_of(const ScanTile* tiles, int ntiles, unsigned long long gb) {
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].bin_base <= gb) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Launch bounds of 4 x 256 threads per SM (64 registers): bins of 4 x 4 pixels run 64-thread CTAs,
// and more of them in flight cover the staging and the FP64 fallbacks (measured 18 % faster).
__global__ void __launch_bounds__(SCAN_THREADS, 4) k_scan(const ScanTile* __restrict__ tiles,
                                                       int ntiles, uint32_t* err,
                                                       unsigned long long* stats) {
  __shared__ ScanSmem sm;
  const unsigned long long gb = blockIdx.x;
  const ScanTile& t = tiles[scan_tile_of(tiles, ntiles, gb)];
  const uint32_t bin = static_cast<uint32_t>(gb - t.bin_base);
  const uint32_t a = t.spp;
  const uint32_t tid = threadIdx.x;
  const ScanRay R = scan_ray(t, bin, tid);
  const uint32_t px = R.px, py = R.py, sx = R.sx, sy = R.sy, st = R.st;
  const bool active = R.active;
  const float oxh = R.oxh, oxl = R.oxl, oyh = R.oyh, oyl = R.oyl;
  long long Lfix = 0;  // chord sum (sigma-weighted when per crystal), 2^-40 um units
  uint32_t nh = 0, nfb = 0;
  const uint32_t b0 = min(t.bin_off[bin], t.items_cap), b1 = min(t.bin_off[bin + 1], t.items_cap);
  const bool per_crystal = t.sigma_c != nullptr;
  for (uint32_t base = b0; base < b1; base += SCAN_CH) {
    const uint32_t cnt = min(static_cast<uint32_t>(SCAN_CH), b1 - base);
    __syncthreads();
    for (uint32_t c = tid; c < cnt; c += blockDim.x)
      stage_crystal(t, sm, c, t.bin_items[base + c], R.bxh, R.bxl, R.byh, R.byl);
    __syncthreads();
    if (!active) continue;
    for (uint32_t c = 0; c < cnt; ++c) {
      float chord;
      const bool hit = scan_pair(t, sm, c, oxh, oxl, oyh, oyl, px, py, sx, sy, chord, nfb);
      if (hit) {
        ++nh;
        const float v = per_crystal ? sm.sig[c] * fmaxf(chord, 0.0f) : fmaxf(chord, 0.0f);
        Lfix += fix40(v);
      }
    }
  }
  float T = 1.0f;
  if (active) {
    // Lfix * 2^-40 rounded once to float (the conversion rounds, the power-of-two scale is exact).
    const float L = u64_to_float_rn(static_cast<unsigned long long>(Lfix)) * 0x1p-40f;
    T = per_crystal ? expf(-L) : expf(-t.sigma * L);
    if (t.ray_hits) t.ray_hits[(static_cast<size_t>(py) * t.w + px) * a + st] = static_cast<uint16_t>(min(nh, 65535u));
  }
  sm.T[tid] = f2d_exact(T);
  __syncthreads();
  // Per pixel: thread p finishes the bin's p-th pixel, so the FP64 work runs on consecutive lanes
  // (a pixel's strata are a consecutive threads; one thread in a per pixel would leave most lanes
  // of each FP64 instruction idle on GB300's narrow FP64 pipe).
  for (uint32_t p = tid; p * a < blockDim.x; p += blockDim.x) {
    const uint32_t bx = bin % t.nbx, by = bin / t.nbx;
    const uint32_t qx = bx * t.bin_px + p % t.bin_px, qy = by * t.bin_px + p / t.bin_px;
    if (p >= t.bin_px * t.bin_px || qx >= t.w || qy >= t.h) continue;
    // FP64 mean over strata in the reference's order (sy, sx), then f32 (transmittance.rs:142).
    double acc = 0.0;
    for (uint32_t k = 0; k < a; ++k) acc = __dadd_rn(acc, sm.T[p * a + k]);
    // Division by a power of two is the multiplication by its exact reciprocal.
    const float mean = (float)((a & (a - 1)) == 0 ? __dmul_rn(acc, 1.0 / static_cast<double>(a))
                                                   : __ddiv_rn(acc, static_cast<double>(a)));
    const size_t idx = static_cast<size_t>(qy) * t.w + qx;
    float v;
    if (t.mode == 0) {
      v = mean;
    } else if (t.mode == 1) {
      v = 1.0f - mean;
    } else {
      const float tt = fmaxf(mean, 1e-4f);
      v = fminf(fmaxf(-log10f(tt) / 3.0f, 0.0f), 1.0f);
    }
    if (t.out) t.out[idx] = v;
    if (t.image8) t.image8[idx] = static_cast<uint8_t>(rintf(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f));
    // The mean transmittance; launch_density turns it into the density in a pass of its own.
    if (t.d_neg) t.d_neg[idx] = mean;
  }
  if (stats) {
    unsigned long long f = nfb, hsum = nh;
    for (int o = 16; o > 0; o >>= 1) {
      f += __shfl_down_sync(0xffffffffu, f, o);
      hsum += __shfl_down_sync(0xffffffffu, hsum, o);
    }
    if ((tid & 31) == 0) {
      if (f) atomicAdd(&stats[1], f);
      if (hsum) atomicAdd(&stats[2], hsum);
    }
  }
}

// Adjoint of k_scan with respect to the per-crystal opacities (single tile).  The forward is
// recomputed from the developed mask: pass 1 forms each ray's optical depth exactly as k_scan
// does, pass 2 re-stages the bin's crystals and adds w[p] / spp * T_ray * chord_s for every hit to
// a per-crystal FP64 sum in shared memory, flushed with one global atomic per staged crystal.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_adjoint(const ScanTile* __restrict__ tiles,
                                                               const float* __restrict__ wpx,
                                                               double* __restrict__ g) {
  __shared__ ScanSmem sm;
  __shared__ double gsum[SCAN_CH];
  const ScanTile& t = tiles[0];
  const uint32_t bin = blockIdx.x;
  const uint32_t a = t.spp;
  const uint32_t tid = threadIdx.x;
  const ScanRay R = scan_ray(t, bin, tid);
  const uint32_t b0 = min(t.bin_off[bin], t.items_cap), b1 = min(t.bin_off[bin + 1], t.items_cap);
  const bool per_crystal = t.sigma_c != nullptr;
  uint32_t nfb = 0;
  long long Lfix = 0;
  for (uint32_t base = b0; base < b1; base += SCAN_CH) {
    const uint32_t cnt = min(static_cast<uint32_t>(SCAN_CH), b1 - base);
    __syncthreads();
    for (uint32_t c = tid; c < cnt; c += blockDim.x)
      stage_crystal(t, sm, c, t.bin_items[base + c], R.bxh, R.bxl, R.byh, R.byl);
    __syncthreads();
    if (!R.active) continue;
    for (uint32_t c = 0; c < cnt; ++c) {
      float chord;
      if (scan_pair(t, sm, c, R.oxh, R.oxl, R.oyh, R.oyl, R.px, R.py, R.sx, R.sy, chord, nfb)) {
        const float v = per_crystal ? sm.sig[c] * fmaxf(chord, 0.0f) : fmaxf(chord, 0.0f);
        Lfix += fix40(v);
      }
    }
  }
  float coef = 0.0f;
  if (R.active) {
    const float L = u64_to_float_rn(static_cast<unsigned long long>(Lfix)) * 0x1p-40f;  // as in k_scan
    const float T = per_crystal ? expf(-L) : expf(-t.sigma * L);
    coef = wpx[static_cast<size_t>(R.py) * t.w + R.px] / static_cast<float>(a) * T;
  }
  for (uint32_t base = b0; base < b1; base += SCAN_CH) {
    const uint32_t cnt = min(static_cast<uint32_t>(SCAN_CH), b1 - base);
    __syncthreads();
    for (uint32_t c = tid; c < cnt; c += blockDim.x) {
      stage_crystal(t, sm, c, t.bin_items[base + c], R.bxh, R.bxl, R.byh, R.byl);
      gsum[c] = 0.0;
    }
    __syncthreads();
    if (R.active && coef != 0.0f) {
      for (uint32_t c = 0; c < cnt; ++c) {
        float chord;
        if (scan_pair(t, sm, c, R.oxh, R.oxl, R.oyh, R.oyl, R.px, R.py, R.sx, R.sy, chord, nfb))
          atomicAdd(&gsum[c], static_cast<double>(coef) * static_cast<double>(fmaxf(chord, 0.0f)));
      }
    }
    __syncthreads();
    for (uint32_t c = tid; c < cnt; c += blockDim.x)
      if (gsum[c] != 0.0) atomicAdd(&g[sm.s[c]], gsum[c]);
  }
}

// d = -log10(clamp(T, 1e-4, 1)) + 0.05 in FP64 (image_pipeline.rs:1007-1011), in place over the
// pixels' mean transmittance.  A pass of its own so that every lane of a warp converts a pixel:
// inside k_scan only one thread per pixel (of spp) would, and each FP64 instruction would occupy
// GB300's narrow FP64 pipe for a whole warp.
__global__ void k_density(float* __restrict__ d, unsigned long long n) {
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += stride) {
    const double tc = fmin(fmax(static_cast<double>(d[i]), 1e-4), 1.0);
    d[i] = static_cast<float>(-log10(tc) + 0.05);
  }
}

void launch_density(float* d, unsigned long long n, cudaStream_t st) {
  if (n == 0) return;
  k_density<<<static_cast<unsigned>(std::min<unsigned long long>(grid_for(n, 256), 152ull * 16)), 256, 0, st>>>(d, n);
  FG_CUDA(cudaGetLastError());
}

void launch_scan(const ScanTile* tiles, int ntiles, unsigned long long nbins, unsigned threads, uint32_t* err,
                 unsigned long long* stats, cudaStream_t st) {
  if (nbins == 0) return;
  k_scan<<<static_cast<unsigned>(nbins), threads, 0, st>>>(tiles, ntiles, err, stats);
  FG_CUDA(cudaGetLastError());
}

// Chooses the bin edge so one CTA holds bin_px^2 pixels of `spp` strata.
uint32_t scan_bin_px(uint32_t spp) {
  uint32_t b = 1;
  while ((b + 1) * (b + 1) * spp <= SCAN_THREADS) ++b;
  return b;
}

// Bins the developed crystals of an emulsion for a scan: descriptor, bin offsets and lists on the
// device (shared by the forward scan and its adjoint).
struct ScanPlan {
  ScanTile t{};
  RTreeBufs tree;             // the reference tree over the developed crystals
  DBuf<uint32_t> tree_list;
  DBuf<ScanPrep> prep;
  DBuf<uint32_t> cnt, off, cur, items;
  DBuf<ScanTile> td;
  unsigned nbins = 0, threads = 0;
};

static void plan_scan(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
                      const float* sigma_sorted, const ScanOut& out, ScanPlan& P) {
  cudaStream_t st = e->stream;
  const uint32_t spp_req = std::max<uint32_t>(cfg.samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::lround(std::sqrt(static_cast<double>(spp_req))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  FG_REQUIRE(a <= SCAN_THREADS, "samples_per_pixel too large (at most 256 strata)");
  FG_REQUIRE(cfg.width_px > 0 && cfg.height_px > 0, "scan size must be positive");
  build_emulsion_tree(e, em, true, P.tree, P.tree_list);
  ScanTile& t = P.t;
  t = ScanTile{};
  t.lbox64 = P.tree.box64.p;
  t.leafof = P.tree.leafof.p;
  t.a = em->a.p;
  t.q = em->q.p;
  t.d = em->d.p;
  t.pos64 = em->has64 ? em->pos64.p : nullptr;
  t.dims64 = em->has64 ? em->dims64.p : nullptr;
  t.quat64 = em->has64 ? em->quat64.p : nullptr;
  t.developed = em->developed.p;
  t.exp64 = em->exp64.p;
  t.sigma_c = sigma_sorted;
  t.out = out.out;
  t.image8 = out.image8;
  t.d_neg = out.d_neg;
  t.ray_hits = out.ray_hits;
  t.pw = em->cfg.width / static_cast<double>(cfg.width_px);
  t.ph = em->cfg.height / static_cast<double>(cfg.height_px);
  t.z0 = em->cfg.depth + 0.1;
  t.seed = seed;
  t.bin_base = 0;
  t.w = cfg.width_px;
  t.h = cfg.height_px;
  t.g = g;
  t.spp = a;
  t.bin_px = scan_bin_px(a);
  t.nbx = (t.w + t.bin_px - 1) / t.bin_px;
  t.nby = (t.h + t.bin_px - 1) / t.bin_px;
  t.n = em->n;
  t.sigma = static_cast<float>(cfg.silver_opacity);
  t.mode = cfg.mode;
  set_jitter_units(t);
  const size_t nbins = static_cast<size_t>(t.nbx) * t.nby;
  FG_REQUIRE(nbins < 0x80000000ull, "scan too large");
  P.nbins = static_cast<unsigned>(nbins);
  P.cnt.alloc(nbins + 1, st);
  P.off.alloc(nbins + 1, st);
  P.cur.alloc(nbins, st);
  FG_CUDA(cudaMemsetAsync(P.cnt.p, 0, (nbins + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(P.cur.p, 0, nbins * sizeof(uint32_t), st));
  if (em->n) k_bin_count<<<grid_for(em->n, 256), 256, 0, st>>>(t, P.cnt.p);
  exclusive_scan_u32(P.cnt.p, P.off.p, nbins + 1, st);
  uint32_t total = 0;
  FG_CUDA(cudaMemcpyAsync(&total, P.off.p + nbins, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  P.items.alloc(std::max<uint32_t>(total, 1), st);
  if (em->n) k_bin_fill<<<grid_for(em->n, 256), 256, 0, st>>>(t, P.off.p, P.cur.p, P.items.p);
  t.bin_off = P.off.p;
  t.bin_items = P.items.p;
  t.items_cap = total;
  t.slot_base = 0;
  P.prep.alloc(std::max<uint32_t>(em->n, 1), st);
  t.prep = P.prep.p;
  P.td.alloc(1, st);
  FG_CUDA(cudaMemcpyAsync(P.td.p, &t, sizeof(ScanTile), cudaMemcpyHostToDevice, st));
  launch_scan_prep(P.td.p, 1, em->n, P.prep.p, st);
  // Whole warps only: the closing reductions shuffle across all 32 lanes.
  P.threads = ((t.bin_px * t.bin_px * a + 31) / 32) * 32;
}

void scan(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
          const float* sigma_sorted, const ScanOut& out) {
  ScanPlan P;
  plan_scan(e, em, cfg, seed, sigma_sorted, out, P);
  k_scan<<<P.nbins, P.threads, 0, e->stream>>>(P.td.p, 1, e->d_err, e->d_stats);
  FG_CUDA(cudaGetLastError());
  if (out.d_neg) launch_density(out.d_neg, static_cast<unsigned long long>(cfg.width_px) * cfg.height_px, e->stream);
  FG_CUDA(cudaStreamSynchronize(e->stream));
}

// Adjoint of the scan with respect to the per-crystal opacities: g[s] += sum over the rays of
// pixel p of w[p] / spp * T_ray * chord_s (w = dL/dT of the pixel, T_ray the ray's transmittance).
void scan_adjoint(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
                  const float* sigma_sorted, const float* wpx, double* g_sorted) {
  ScanPlan P;
  plan_scan(e, em, cfg, seed, sigma_sorted, ScanOut{}, P);
  k_scan_adjoint<<<P.nbins, P.threads, 0, e->stream>>>(P.td.p, wpx, g_sorted);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(e->stream));
}

}  // namespace fg
