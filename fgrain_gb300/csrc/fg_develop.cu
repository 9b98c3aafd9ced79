// Development (development.rs:59-188) on the device: threshold the latent counts into the
// developed mask, then group touching developed crystals into clumps.
//
// The reference walks a breadth-first search from each undeveloped-yet-unvisited crystal in
// index order.  Its clumps are exactly the connected components of the symmetric "touch" graph
// |p_i - p_j|^2 <= ((r_i fe + r_j fe) prox)^2 over developed crystals (every touch test uses the
// base expansion fe; the boost is applied after a component is complete).  Here each developed
// crystal finds its touching neighbours through a box query on the emulsion's reference tree
// (the four-wide walk records, fg_rtree.cuh) and links them with a
// lock-free union-find.  Clump ids follow the reference's numbering: components ranked by their
// smallest crystal index.  Touch decisions are exact: an FP32 test with an error margin, and the
// reference's FP64 expression when the margin is too thin to decide.
#include <cstring>

#include "fg_internal.h"

namespace fg {

struct DevCounters {
  unsigned long long developed;
  unsigned long long clumps;
  unsigned long long max_size;
  unsigned long long fallbacks;
};

__global__ void k_threshold(const uint32_t* counts, uint32_t n, uint32_t thr, double fe,
                            uint8_t* developed, double* exp64, int* parent, DevCounters* dc) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const bool dv = counts[s] >= thr;
  developed[s] = dv ? 1 : 0;
  exp64[s] = dv ? fe : 0.0;
  parent[s] = static_cast<int>(s);
  const unsigned act = __activemask();
  const unsigned ball = __ballot_sync(act, dv);
  if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(act) - 1) && ball)
    atomicAdd(&dc->developed, static_cast<unsigned long long>(__popc(ball)));
}

__device__ __forceinline__ int uf_find(int* parent, int x, uint32_t* err) {
  for (int it = 0; it < (1 << 22); ++it) {
    const int p = __ldcg(&parent[x]);
    if (p == x) return x;
    const int gp = __ldcg(&parent[p]);
    if (gp != p) atomicCAS(&parent[x], p, gp);  // path halving
    x = gp;
  }
  atomicOr(err, ERR_SPIN_LIMIT);
  return x;
}

__device__ __forceinline__ void uf_unite(int* parent, int a, int b, uint32_t* err) {
  for (int it = 0; it < (1 << 20); ++it) {
    a = uf_find(parent, a, err);
    b = uf_find(parent, b, err);
    if (a == b) return;
    if (a > b) { const int t = a; a = b; b = t; }
    const int old = atomicCAS(&parent[b], b, a);
    if (old == b) return;
    b = old;
  }
  atomicOr(err, ERR_SPIN_LIMIT);
}

__global__ void k_link(CrystalsView cv, const Node4* __restrict__ rec, uint32_t nrec, const uint2* __restrict__ rleaf,
                       uint32_t nleaf, const uint32_t* __restrict__ ridx, uint32_t n,
                       const uint8_t* __restrict__ developed, double fe, double prox,
                       double max_base, int* parent, DevCounters* dc, uint32_t* err) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !developed[s]) return;
  const float4 a = cv.a[s], d = cv.d[s];
  const double ms = cv.dims64 ? fmax(fmax(cv.dims64[3 * s], cv.dims64[3 * s + 1]), cv.dims64[3 * s + 2])
                              : (double)fmaxf(fmaxf(d.x, d.y), d.z);
  const double rc = __dmul_rn(ms, fe);
  const double search = __dmul_rn(__dadd_rn(rc, __dmul_rn(max_base, fe)), prox);
  const float R = (float)search * 1.0001f + 1e-3f;
  const float3 lo = make_float3(a.x - R, a.y - R, a.z - R), hi = make_float3(a.x + R, a.y + R, a.z + R);
  const float fef = (float)fe, proxf = (float)prox;
  const float rcf = fmaxf(fmaxf(d.x, d.y), d.z) * fef;
  unsigned long long fb = 0;
  auto test = [&](uint32_t j) {
    if (j <= s || j >= n || !developed[j]) return;
    const float4 aj = cv.a[j], dj = cv.d[j];
    const float dx = aj.x - a.x, dy = aj.y - a.y, dz = aj.z - a.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float touch = (rcf + fmaxf(fmaxf(dj.x, dj.y), dj.z) * fef) * proxf;
    const float t2 = touch * touch;
    // Positions rounded to FP32 move |dp|^2 by at most ~4 ulp(|p|) |dp|; 1e-3 relative + an
    // absolute term bounds that, and everything else, generously.
    const float pmag = fabsf(a.x) + fabsf(a.y) + fabsf(a.z);
    const float margin = 1e-3f * t2 + 4e-7f * pmag * (touch + 1.0f);
    bool touch_hit;
    if (d2 < t2 - margin) {
      touch_hit = true;
    } else if (d2 > t2 + margin) {
      touch_hit = false;
    } else {
      ++fb;
      const Crystal64 ci = load64(cv, s), cj = load64(cv, j);
      const double rn = __dmul_rn(fmax(fmax(cj.dims.x, cj.dims.y), cj.dims.z), fe);
      const double tt = __dmul_rn(__dadd_rn(rc, rn), prox);
      const D3 df = dsub3(cj.pos, ci.pos);
      touch_hit = ddot(df, df) <= __dmul_rn(tt, tt);
    }
    if (touch_hit) uf_unite(parent, static_cast<int>(s), static_cast<int>(j), err);
  };
  rt_walk4_box(rec, lo, hi, nrec, err, [&](uint32_t leaf) {
    if (!index_ok(leaf < nleaf, err, SITE_LEAF, leaf, nleaf)) return;
    const uint2 L = rleaf[leaf];
    if (!index_ok(L.x + L.y <= n, err, SITE_LEAF, L.x, L.y)) return;
    for (uint32_t k = 0; k < L.y; ++k) test(ridx[L.x + k]);
  });
  if (fb) atomicAdd(&dc->fallbacks, fb);
}

__global__ void k_roots(uint32_t n, const uint8_t* developed, int* parent, const uint32_t* s2id,
                        uint32_t* size, uint32_t* minid, uint32_t* err) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !developed[s]) return;
  const int r = uf_find(parent, static_cast<int>(s), err);
  parent[s] = r;
  atomicAdd(&size[r], 1u);
  atomicMin(&minid[r], s2id ? s2id[s] : s);
}

__global__ void k_flags(uint32_t n, const uint8_t* developed, const int* parent, const uint32_t* s2id,
                        const uint32_t* size, const uint32_t* minid, uint32_t* flag_by_id,
                        DevCounters* dc) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  // Clumps are numbered by their smallest crystal index (the reference's BFS start order), so
  // each component flags its minimum id; a prefix sum over ids then ranks them.
  const bool root = developed[s] && parent[s] == static_cast<int>(s);
  if (root) flag_by_id[minid[s]] = 1u;
  const unsigned act = __activemask();
  const unsigned ball = __ballot_sync(act, root);
  const unsigned mx = __reduce_max_sync(act, root ? size[s] : 0u);
  if ((threadIdx.x & 31) == static_cast<unsigned>(__ffs(act) - 1) && ball) {
    atomicAdd(&dc->clumps, static_cast<unsigned long long>(__popc(ball)));
    atomicMax(&dc->max_size, static_cast<unsigned long long>(mx));
  }
  (void)s2id;
}

__global__ void k_finalize(uint32_t n, const uint8_t* developed, const int* parent,
                           const uint32_t* s2id, const uint32_t* size, const uint32_t* minid,
                           const uint32_t* rank_by_id, double fe, double* exp64, float* exp32,
                           int64_t* clump_by_id) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t id = s2id ? s2id[s] : s;
  if (!developed[s]) {
    exp64[s] = 0.0;
    exp32[s] = 0.0f;
    clump_by_id[id] = -1;
    return;
  }
  const int r = parent[s];
  const uint32_t sz = size[r];
  double e = fe;
  if (sz > 1) {
    const double boost = __dadd_rn(1.15, __dmul_rn(0.18, static_cast<double>((sz < 6 ? sz : 6) - 1)));
    e = __dmul_rn(fe, boost);
  }
  exp64[s] = e;
  exp32[s] = static_cast<float>(e);
  clump_by_id[id] = static_cast<int64_t>(rank_by_id[minid[r]]);
}

__global__ void k_maxdim(CrystalsView cv, uint32_t n, unsigned long long* out) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (s < n) {
    if (cv.dims64) {
      m = fmax(fmax(cv.dims64[3 * s], cv.dims64[3 * s + 1]), cv.dims64[3 * s + 2]);
    } else {
      const float4 d = cv.d[s];
      m = (double)fmaxf(fmaxf(d.x, d.y), d.z);
    }
  }
  // Non-negative doubles order like their bit patterns.
  atomicMax(out, static_cast<unsigned long long>(__double_as_longlong(m)));
}

void develop(fg_engine* e, fg_emulsion* em, const fg_dev_cfg& cfg, fg_dev_report* rep) {
  cudaStream_t st = e->stream;
  const uint32_t n = em->n;
  fg_dev_report r{};
  r.total_crystals = n;
  if (n == 0) {
    if (rep) *rep = r;
    return;
  }
  DBuf<DevCounters> dc(1, st);
  DBuf<int> parent(n, st);
  DBuf<uint32_t> size(n, st), minid(n, st), flag(n, st), rank(n, st);
  DBuf<unsigned long long> mb(1, st);
  FG_CUDA(cudaMemsetAsync(dc.p, 0, sizeof(DevCounters), st));
  FG_CUDA(cudaMemsetAsync(size.p, 0, n * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(minid.p, 0xff, n * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(flag.p, 0, n * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(mb.p, 0, sizeof(unsigned long long), st));
  const unsigned G = grid_for(n, 256);
  const uint32_t* s2id = em->h_s2id.empty() ? nullptr : em->sorted_to_id.p;
  k_maxdim<<<G, 256, 0, st>>>(em->view(), n, mb.p);
  k_threshold<<<G, 256, 0, st>>>(em->counts.p, n, cfg.threshold_photons, cfg.filament_expansion,
                                 em->developed.p, em->exp64.p, parent.p, dc.p);
  unsigned long long mbits = 0;
  FG_CUDA(cudaMemcpyAsync(&mbits, mb.p, sizeof(mbits), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  double max_base;
  std::memcpy(&max_base, &mbits, sizeof(double));
  k_link<<<G, 256, 0, st>>>(em->view(), em->rt.rnode.p, static_cast<uint32_t>(em->rt.R), em->rt.rleaf.p,
                            static_cast<uint32_t>(em->rt.N), em->rt.ridx.p, n, em->developed.p, cfg.filament_expansion,
                            cfg.clumping_proximity_factor, max_base, parent.p, dc.p, e->d_err);
  k_roots<<<G, 256, 0, st>>>(n, em->developed.p, parent.p, s2id, size.p, minid.p, e->d_err);
  k_flags<<<G, 256, 0, st>>>(n, em->developed.p, parent.p, s2id, size.p, minid.p, flag.p, dc.p);
  exclusive_scan_u32(flag.p, rank.p, n, st);
  k_finalize<<<G, 256, 0, st>>>(n, em->developed.p, parent.p, s2id, size.p, minid.p, rank.p,
                                cfg.filament_expansion, em->exp64.p, em->exp32.p, em->clump.p);
  FG_CUDA(cudaGetLastError());
  DevCounters h{};
  FG_CUDA(cudaMemcpyAsync(&h, dc.p, sizeof(h), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  r.developed_crystals = h.developed;
  r.fixed_crystals = n - h.developed;
  r.total_clumps = h.clumps;
  r.max_clump_size = h.max_size;
  r.avg_clump_size = h.clumps ? static_cast<double>(h.developed) / static_cast<double>(h.clumps) : 0.0;
  e->timings.developed = h.developed;
  e->timings.fallbacks += h.fallbacks;
  if (rep) *rep = r;
}

}  // namespace fg
