// Transmittance scan kernels: binning of developed crystals and the binned scan itself.
#include "fg_internal.h"
#include "fg_scan.cuh"

namespace fg {

// Bin range of crystal s's own box (max_dim * expansion) in one axis.
__device__ __forceinline__ void bin_range(float c, float m, float binw, uint32_t nb, uint32_t& b0,
                                          uint32_t& b1) {
  const float lo = (c - m - 1e-3f) / binw, hi = (c + m + 1e-3f) / binw;
  const float fl = fminf(fmaxf(floorf(lo), 0.0f), (float)(nb - 1));
  const float fh = fminf(fmaxf(floorf(hi), 0.0f), (float)(nb - 1));
  b0 = static_cast<uint32_t>(fl);
  b1 = static_cast<uint32_t>(fh);
}

__device__ __forceinline__ float own_half(const ScanTile& t, uint32_t s) {
  const float4 d = t.d[s];
  return fmaxf(fmaxf(d.x, d.y), d.z) * (float)t.exp64[s];
}

__global__ void k_bin_count(ScanTile t, uint32_t* cnt) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= t.n || !t.developed[s]) return;
  const float4 a = t.a[s];
  const float m = own_half(t, s) * 1.0001f;
  uint32_t x0, x1, y0, y1;
  bin_range(a.x, m, (float)(t.bin_px * t.pw), t.nbx, x0, x1);
  bin_range(a.y, m, (float)(t.bin_px * t.ph), t.nby, y0, y1);
  for (uint32_t by = y0; by <= y1; ++by)
    for (uint32_t bx = x0; bx <= x1; ++bx) atomicAdd(&cnt[by * t.nbx + bx], 1u);
}

__global__ void k_bin_fill(ScanTile t, const uint32_t* off, uint32_t* cursor, uint32_t* items) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= t.n || !t.developed[s]) return;
  const float4 a = t.a[s];
  const float m = own_half(t, s) * 1.0001f;
  uint32_t x0, x1, y0, y1;
  bin_range(a.x, m, (float)(t.bin_px * t.pw), t.nbx, x0, x1);
  bin_range(a.y, m, (float)(t.bin_px * t.ph), t.nby, y0, y1);
  for (uint32_t by = y0; by <= y1; ++by)
    for (uint32_t bx = x0; bx <= x1; ++bx) {
      const uint32_t b = by * t.nbx + bx;
      items[off[b] + atomicAdd(&cursor[b], 1u)] = s;
    }
}

// Shared-memory image of a staged crystal (index c of the current chunk).
struct ScanSmem {
  float cx[SCAN_CH], cy[SCAN_CH], m[SCAN_CH], delta[SCAN_CH], err[SCAN_CH], sig[SCAN_CH];
  float g[12][SCAN_CH];
  int s[SCAN_CH];
  int type[SCAN_CH];
  double T[SCAN_THREADS];
};

// Stages crystal s for vertical rays relative to the bin corner (bx0, by0) (FP64 corner).
__device__ __forceinline__ void stage_crystal(const ScanTile& t, ScanSmem& sm, int c, uint32_t s,
                                              double bx0, double by0) {
  const float4 a = t.a[s], q = t.q[s], d = t.d[s];
  double px, py, pz, mdim;
  if (t.pos64) {
    px = t.pos64[3 * s];
    py = t.pos64[3 * s + 1];
    pz = t.pos64[3 * s + 2];
    mdim = fmax(fmax(t.dims64[3 * s], t.dims64[3 * s + 1]), t.dims64[3 * s + 2]);
  } else {
    px = a.x; py = a.y; pz = a.z;
    mdim = (double)fmaxf(fmaxf(d.x, d.y), d.z);
  }
  const double e64 = t.exp64[s];
  const float e = (float)e64;
  const float m = (float)__dmul_rn(mdim, e64);
  sm.cx[c] = (float)(px - bx0);
  sm.cy[c] = (float)(py - by0);
  sm.m[c] = m;
  sm.delta[c] = (float)(t.z0 - pz);
  sm.sig[c] = t.sigma_c ? t.sigma_c[s] : t.sigma;
  sm.s[c] = static_cast<int>(s);
  const float x = q.x, y = q.y, z = q.z, w = q.w;
  // world = R local + p, so local_i = R_0i dx + R_1i dy + R_2i dz: rows 0..2 of R.
  const float R0[3] = {1.f - 2.f * (y * y + z * z), 2.f * (x * y - z * w), 2.f * (x * z + y * w)};
  const float R1[3] = {2.f * (x * y + z * w), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - x * w)};
  const float R2[3] = {2.f * (x * z - y * w), 2.f * (y * z + x * w), 1.f - 2.f * (x * x + y * y)};
  const float D[3] = {d.x * e, d.y * e, d.z * e};
  const float eps = 5.9604645e-8f;
  const float dlt = SCAN_DELTA;
  if (morph_of(d) == 0) {
    sm.type[c] = 0;
    float invmax = 0.0f, Dmax = fmaxf(fmaxf(D[0], D[1]), D[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      sm.g[i][c] = R0[i];
      sm.g[3 + i][c] = R1[i];
      const float inv = 1.0f / (-R2[i]);
      sm.g[6 + i][c] = inv;
      sm.g[9 + i][c] = D[i];
      invmax = fmaxf(invmax, fabsf(inv));
    }
    const float Tmax = (Dmax + 2.0f * m) * invmax;
    float E = 4.0f * ((24.0f * eps * m + 2.0f * dlt + 2.0f * eps * Dmax) * invmax +
                      eps * Tmax * (12.0f * invmax + 2.0f));
    if (!(E < 1e30f)) E = INFINITY;  // axis-parallel faces: always decide in FP64
    sm.err[c] = E;
  } else {
    sm.type[c] = 1;
    float A = 0.0f, Dmin = fminf(fminf(D[0], D[1]), D[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      sm.g[i][c] = R0[i] / D[i];
      sm.g[3 + i][c] = R1[i] / D[i];
      const float ei = -R2[i] / D[i];
      sm.g[6 + i][c] = ei;
      A += ei * ei;
    }
    sm.g[9][c] = A;
    sm.g[10][c] = 1.0f / A;
    sm.g[11][c] = 0.0f;
    const float Pmax = 1.4142136f * m / Dmin;
    const float dP = 1.7320508f * (28.0f * eps * m + 2.0f * dlt) / Dmin;
    const float de = 1.7320508f * 14.0f * eps / Dmin;
    const float sA = sqrtf(A);
    sm.err[c] = 2.0f * (4.0f * A * Pmax * dP + 4.0f * sA * (Pmax * Pmax + 1.0f) * de +
                        6.0f * eps * A * (2.0f * Pmax * Pmax + 1.0f));
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan(const ScanTile* __restrict__ tiles,
                                                       int ntiles, uint32_t* err,
                                                       unsigned long long* stats) {
  __shared__ ScanSmem sm;
  // Tile of this bin (last tile whose first bin <= blockIdx.x).
  int lo = 0, hi = ntiles - 1;
  const unsigned long long gb = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].bin_base <= gb) lo = mid; else hi = mid - 1;
  }
  const ScanTile& t = tiles[lo];
  const uint32_t bin = static_cast<uint32_t>(gb - t.bin_base);
  const uint32_t bx = bin % t.nbx, by = bin / t.nbx;
  const uint32_t a = t.spp;
  const uint32_t tid = threadIdx.x;
  const uint32_t pix = tid / a, st = tid % a;
  const uint32_t lx = pix % t.bin_px, ly = pix / t.bin_px;
  const uint32_t px = bx * t.bin_px + lx, py = by * t.bin_px + ly;
  const bool active = pix < t.bin_px * t.bin_px && px < t.w && py < t.h;
  const uint32_t sx = st % t.g, sy = st / t.g;
  const double bx0 = __dmul_rn(static_cast<double>(bx * t.bin_px), t.pw);
  const double by0 = __dmul_rn(static_cast<double>(by * t.bin_px), t.ph);
  // FP32 ray position relative to the bin corner.
  float ox = 0.0f, oy = 0.0f;
  P4 r{};
  if (active) {
    const uint64_t ps = t.seed + static_cast<uint64_t>(px) * 0x9E3779B97F4A7C15ull +
                        static_cast<uint64_t>(py) * 0xC6A4A7935BD1E995ull;
    r = philox(sy * t.g + sx, 0, 0, TAG_SCAN, static_cast<uint32_t>(ps), static_cast<uint32_t>(ps >> 32));
    const float gf = (float)t.g;
    ox = ((float)lx + ((float)sx + uf(r.x)) / gf) * (float)t.pw;
    oy = ((float)ly + ((float)sy + uf(r.y)) / gf) * (float)t.ph;
  }
  long long Lfix = 0;  // sum of sigma-weighted chords, 2^-40 um units (sigma folded in when per-crystal)
  uint32_t nh = 0, nfb = 0;
  const uint32_t b0 = t.bin_off[bin], b1 = t.bin_off[bin + 1];
  const float EB = 2.0f * SCAN_DELTA;
  const bool per_crystal = t.sigma_c != nullptr;
  for (uint32_t base = b0; base < b1; base += SCAN_CH) {
    const uint32_t cnt = min(static_cast<uint32_t>(SCAN_CH), b1 - base);
    __syncthreads();
    for (uint32_t c = tid; c < cnt; c += blockDim.x) stage_crystal(t, sm, c, t.bin_items[base + c], bx0, by0);
    __syncthreads();
    if (!active) continue;
    for (uint32_t c = 0; c < cnt; ++c) {
      const float dx = ox - sm.cx[c], dy = oy - sm.cy[c];
      const float m = sm.m[c];
      const float mx = m - fabsf(dx), my = m - fabsf(dy), mz = sm.delta[c] + m;
      if (mx < -EB || my < -EB || mz < -EB) continue;
      bool amb = mx <= EB || my <= EB || mz <= EB;
      bool hit = false;
      float chord = 0.0f;
      if (!amb) {
        const float E = sm.err[c];
        const float delta = sm.delta[c];
        if (sm.type[c] == 0) {
          float tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            const float lo_i = sm.g[i][c] * dx + sm.g[3 + i][c] * dy;
            const float inv = sm.g[6 + i][c], D = sm.g[9 + i][c];
            const float t1 = (-D - lo_i) * inv, t2 = (D - lo_i) * inv;
            tmin = fmaxf(tmin, fminf(t1, t2));
            tmax = fminf(tmax, fmaxf(t1, t2));
          }
          const float m1 = tmax - tmin, m2 = tmax + delta;
          if (m1 > 2.0f * E && m2 > E + 1e-6f) {
            hit = true;
            chord = tmax - fmaxf(tmin, -delta);
          } else if (!(m1 < -2.0f * E || m2 < -E - 1e-6f)) {
            amb = true;
          }
        } else {
          float P[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) P[i] = sm.g[i][c] * dx + sm.g[3 + i][c] * dy;
          const float A = sm.g[9][c], iA = sm.g[10][c];
          const float qd = P[0] * sm.g[6][c] + P[1] * sm.g[7][c] + P[2] * sm.g[8][c];
          const float C = P[0] * P[0] + P[1] * P[1] + P[2] * P[2] - 1.0f;
          const float wv = qd * qd - A * C;
          if (wv > E) {
            const float sq = sqrtf(wv);
            const float t0 = (-qd - sq) * iA, t1 = (-qd + sq) * iA;
            if (t1 + delta > 1e-4f) {
              hit = true;
              chord = t1 - fmaxf(t0, -delta);
            } else {
              amb = true;  // crystal at or above the scanner origin: let FP64 decide
            }
          } else if (!(wv < -E)) {
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
      if (hit) {
        ++nh;
        const float v = per_crystal ? sm.sig[c] * fmaxf(chord, 0.0f) : fmaxf(chord, 0.0f);
        Lfix += __float2ll_rn(v * 1099511627776.0f);
      }
    }
  }
  float T = 1.0f;
  if (active) {
    const float L = (float)((double)Lfix * 9.094947017729282e-13);
    T = per_crystal ? expf(-L) : expf(-t.sigma * L);
    if (t.ray_hits) t.ray_hits[(static_cast<size_t>(py) * t.w + px) * a + st] = static_cast<uint16_t>(min(nh, 65535u));
  }
  sm.T[tid] = (double)T;
  __syncthreads();
  if (active && st == 0) {
    // FP64 mean over strata in the reference's order (sy, sx), then f32 (transmittance.rs:142).
    double acc = 0.0;
    for (uint32_t k = 0; k < a; ++k) acc = __dadd_rn(acc, sm.T[tid + k]);
    const float mean = (float)__ddiv_rn(acc, (double)a);
    const size_t idx = static_cast<size_t>(py) * t.w + px;
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
    if (t.d_neg) {
      // d = -log10(clamp(T, 1e-4, 1)) + 0.05 in FP64 (image_pipeline.rs:1007-1011).
      const double tc = fmin(fmax((double)mean, 1e-4), 1.0);
      t.d_neg[idx] = (float)(-log10(tc) + 0.05);
    }
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

// Chooses the bin edge so one CTA holds bin_px^2 pixels of `spp` strata.
uint32_t scan_bin_px(uint32_t spp) {
  uint32_t b = 1;
  while ((b + 1) * (b + 1) * spp <= SCAN_THREADS) ++b;
  return b;
}

void scan(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
          const float* sigma_sorted, const ScanOut& out) {
  cudaStream_t st = e->stream;
  const uint32_t spp_req = std::max<uint32_t>(cfg.samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::lround(std::sqrt(static_cast<double>(spp_req))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  FG_REQUIRE(a <= SCAN_THREADS, "samples_per_pixel too large (at most 256 strata)");
  FG_REQUIRE(cfg.width_px > 0 && cfg.height_px > 0, "scan size must be positive");
  ScanTile t{};
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
  const size_t nbins = static_cast<size_t>(t.nbx) * t.nby;
  DBuf<uint32_t> cnt(nbins + 1, st), off(nbins + 1, st), cur(nbins, st);
  FG_CUDA(cudaMemsetAsync(cnt.p, 0, (nbins + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(cur.p, 0, nbins * sizeof(uint32_t), st));
  if (em->n) k_bin_count<<<grid_for(em->n, 256), 256, 0, st>>>(t, cnt.p);
  exclusive_scan_u32(cnt.p, off.p, nbins + 1, st);
  uint32_t total = 0;
  FG_CUDA(cudaMemcpyAsync(&total, off.p + nbins, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  DBuf<uint32_t> items(std::max<uint32_t>(total, 1), st);
  if (em->n) k_bin_fill<<<grid_for(em->n, 256), 256, 0, st>>>(t, off.p, cur.p, items.p);
  t.bin_off = off.p;
  t.bin_items = items.p;
  DBuf<ScanTile> td(1, st);
  FG_CUDA(cudaMemcpyAsync(td.p, &t, sizeof(ScanTile), cudaMemcpyHostToDevice, st));
  k_scan<<<static_cast<unsigned>(nbins), t.bin_px * t.bin_px * a, 0, st>>>(td.p, 1, e->d_err, e->d_stats);
  FG_CUDA(cudaGetLastError());
  FG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace fg
