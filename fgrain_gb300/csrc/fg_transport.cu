// Monte-Carlo photon transport (transport.rs:48-188 and optics.rs:75-196) as a persistent,
// warp-scheduled kernel over one or many tiles, plus the exact replay of recorded segments.
//
// Work: photon ids of all tiles form one index space; each warp takes 32 ids at a time from a
// global counter.  Every draw is a Philox block named by (photon, bounce, slot, tag), so results
// do not depend on which warp or SM traces a photon.  Each segment walks the tile's reference tree
// (fg_rtree.cuh) and absorbs its hits in the reference's traversal order as they are found
// (Beer-Lambert, Bernoulli rounding of 5 E p s latent photons, energy *= max(1 - 0.9 p, 0.05)).
// Counts reach HBM as warp-aggregated atomics.
#include "fg_internal.h"
#include "fg_transport.cuh"

namespace fg {

// ---------------------------------------------------------------------------------------------
// Production kernel.  Every lane carries one photon through its bounces; a lane is in one of five
// states: no photon, a photon between bounces, a bounce walking (fg_transport.cuh: Bounce), a
// walked bounce whose end is pending, or done (the photon queue is spent).  Each loop turn the warp
// does one of two kinds of work:
//   - restart: once WALK_RESTART lanes are idle (or none walks), the walked lanes end their
//     bounces, lanes between bounces begin the next one, and empty lanes take the next photons of
//     the position-ordered queue (which begin their first bounce at once);
//   - otherwise walk: while a walking lane still needs a leaf, walk steps for every walking lane
//     whose leaf queue has room; then every walking lane tests its oldest queued leaf.
// So lanes whose walk ended early wait for a group of restarts, not for the warp's longest walk,
// and the ends and beginnings of bounces still run with many lanes.  Which lane traces a photon,
// and when, never changes its result: its draws are named by (photon, bounce, slot, tag), and its
// leaves are tested in walk order.
// Launch bounds of 4 blocks of 256 per SM (64 registers): the walk is latency-bound.
__global__ void __launch_bounds__(256, 4) k_transport(const TileDesc* __restrict__ tiles, int ntiles,
                                                     unsigned long long total, const uint32_t* __restrict__ order,
                                                     unsigned long long* next, uint32_t* err,
                                                     unsigned long long* stats) {
  constexpr unsigned FULL = 0xffffffffu;
  enum : int { EMPTY_LANE = 0, READY = 1, WALKING = 2, WALKED = 3, DONE = 4 };
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  Photon ph{};
  Bounce w;
  int stack[RT_STACK4];
  int tile = 0;
  int state = EMPTY_LANE;
  unsigned long long my_hits = 0;
  w.cur = WALK_EMPTY;
#pragma unroll
  for (int j = 0; j < WALK_LEAVES; ++j) w.lv[j] = WALK_NONE;
  for (;;) {
    if (state == WALKING && w.cur == WALK_EMPTY && w.lv[0] == WALK_NONE) state = WALKED;
    const unsigned walkm = __ballot_sync(FULL, state == WALKING);
    const unsigned idlem = __ballot_sync(FULL, state != WALKING && state != DONE);
    if (!(walkm | idlem)) break;
    if (!walkm || __popc(idlem) >= WALK_RESTART) {
      if (state == WALKED) {
        my_hits += w.nh;
        state = bounce_end(tiles[tile], ph, w) ? READY : EMPTY_LANE;
      }
      if (state == READY) {
        if (ph.b < tiles[tile].max_bounces) {
          bounce_begin(tiles[tile], ph, w);
          state = WALKING;
        } else {
          state = EMPTY_LANE;
        }
      }
      unsigned need = __ballot_sync(FULL, state == EMPTY_LANE);
      while (need) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(next, static_cast<unsigned long long>(__popc(need)));
        base = __shfl_sync(FULL, base, 0);
        if (state == EMPTY_LANE) {
          const unsigned long long g = base + __popc(need & lt);
          if (g >= total) {
            state = DONE;
          } else {
            unsigned long long gid = order ? order[g] : g;
            if (!index_ok(gid < total, err, SITE_PHOTON_ID, static_cast<uint32_t>(gid), static_cast<uint32_t>(g)))
              gid = g;
            int lo = 0, hi = ntiles - 1;
            while (lo < hi) {
              const int mid = (lo + hi + 1) >> 1;
              if (tiles[mid].photon_base <= gid) lo = mid; else hi = mid - 1;
            }
            tile = lo;
            if (emit_photon(tiles[lo], static_cast<uint32_t>(gid - tiles[lo].photon_base), ph) &&
                ph.b < tiles[lo].max_bounces) {
              bounce_begin(tiles[lo], ph, w);
              state = WALKING;
            }
          }
        }
        need = __ballot_sync(FULL, state == EMPTY_LANE);
      }
      continue;
    }
    for (;;) {
      if (!__any_sync(FULL, state == WALKING && w.cur != WALK_EMPTY && w.lv[0] == WALK_NONE)) break;
      if (state == WALKING && w.cur != WALK_EMPTY && w.lv[WALK_LEAVES - 1] == WALK_NONE)
        walk_step(tiles[tile], w, stack, err);
    }
    if (state == WALKING && w.lv[0] != WALK_NONE) leaf_step(tiles[tile], ph, w, err);
  }
  if (stats) {
    for (int o = 16; o > 0; o >>= 1) my_hits += __shfl_down_sync(FULL, my_hits, o);
    if (lane == 0 && my_hits) atomicAdd(&stats[0], my_hits);
  }
}

// Photon ordering: a counting sort of photon ids by the coarse emission cell (Morton order inside
// each tile), so neighbouring lanes trace neighbouring packets.  Pass 1 (off == null) counts,
// pass 2 scatters.  The order only changes which lane traces a photon, never its result.
__global__ void k_photon_sort(const TileDesc* __restrict__ tiles, int ntiles, unsigned long long total,
                              unsigned long long ncells, uint32_t* cnt, const uint32_t* off, uint32_t* cur,
                              uint32_t* order, uint32_t* err) {
  const unsigned long long gid = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (gid >= total) return;
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].photon_base <= gid) lo = mid; else hi = mid - 1;
  }
  const TileDesc& t = tiles[lo];
  const uint32_t id = static_cast<uint32_t>(gid - t.photon_base);
  const P4 e0 = philox(id, 0, 0, TAG_EMIT, t.k0, t.k1);
  const uint32_t mx = (1u << t.pcell_bits) - 1u;
  const uint32_t cx = min(static_cast<uint32_t>(uf(e0.x) * t.W * (1.0f / PHOTON_CELL_UM)), mx);
  const uint32_t cy = min(static_cast<uint32_t>(uf(e0.y) * t.H * (1.0f / PHOTON_CELL_UM)), mx);
  const uint32_t cell = t.pcell_base + (morton2_spread(cx) | (morton2_spread(cy) << 1));
  if (!index_ok(cell < ncells, err, SITE_PHOTON_CELL, cell, static_cast<uint32_t>(gid))) return;
  if (!off) {
    atomicAdd(&cnt[cell], 1u);
  } else {
    const unsigned long long k = off[cell] + atomicAdd(&cur[cell], 1u);
    if (index_ok(k < total, err, SITE_PHOTON_SLOT, static_cast<uint32_t>(k), cell)) order[k] = static_cast<uint32_t>(gid);
  }
}

void launch_photon_sort(const TileDesc* tiles_dev, int ntiles, unsigned long long total, unsigned long long ncells,
                        uint32_t* cnt, const uint32_t* off, uint32_t* cur, uint32_t* order, uint32_t* err,
                        cudaStream_t st) {
  if (total == 0) return;
  k_photon_sort<<<grid_for(total, 256), 256, 0, st>>>(tiles_dev, ntiles, total, ncells, cnt, off, cur, order, err);
  FG_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------------------------
// Exact replay of recorded segments: the reference walk in FP64 (rt_walk64 over the reference
// tree, whole ray, the reference's stack rule), each leaf crystal tested with the reference's
// geometry in FP64, hits inside the step absorbed in walk order (transport.rs:108-138).  pass 0
// counts hits per segment; pass 1 writes hit ids and adds the latent photons.
struct RtView {
  const double* box64;
  const int2* nchild;
  const int* nsplit;
  const uint32_t* nstart;
  const uint32_t* ncount;
  const uint32_t* ridx;
  uint32_t root;
  uint32_t count;  // elements of the tree (none: nothing to walk)
};

RtView rt_view(const RTreeBufs& B) {
  RtView v;
  v.box64 = B.box64.p;
  v.nchild = B.nchild.p;
  v.nsplit = B.nsplit.p;
  v.nstart = B.nstart.p;
  v.ncount = B.ncount.p;
  v.ridx = B.ridx.p;
  v.root = 1;
  v.count = B.count;
  return v;
}

template <class F>
__device__ __forceinline__ void rt_crystals64(const RtView& rv, D3 o, D3 inv, uint32_t n, uint32_t* err, F&& fn) {
  if (n == 0 || rv.count == 0) return;
  rt_walk64(rv.box64, rv.nchild, rv.nsplit, rv.root, o, inv, [&](uint32_t leaf) {
    const uint32_t st = rv.nstart[leaf], cn = rv.ncount[leaf];
    for (uint32_t k = 0; k < cn; ++k) {
      const uint32_t s = rv.ridx[st + k];
      if (index_ok(s < n, err, SITE_LEAF, s, n)) fn(s);
    }
  });
}

__global__ void k_replay_segments(const fg_segment* __restrict__ segs, uint32_t nseg, CrystalsView cv, RtView rv,
                                  const uint32_t* __restrict__ s2id, uint32_t n, double alpha, uint32_t k0,
                                  uint32_t k1, int pass, uint32_t* seg_count, const uint32_t* offsets, uint32_t* ids,
                                  uint32_t id_cap, uint32_t* counts, uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nseg || n == 0) return;
  const fg_segment g = segs[i];
  const D3 o = d3(g.origin[0], g.origin[1], g.origin[2]);
  const D3 d = d3(g.dir[0], g.dir[1], g.dir[2]);
  const D3 inv = d3(__ddiv_rn(1.0, d.x), __ddiv_rn(1.0, d.y), __ddiv_rn(1.0, d.z));
  double E = g.energy;
  const uint32_t base = pass ? offsets[i] : 0u;
  uint32_t nh = 0;
  P4 r{};
  rt_crystals64(rv, o, inv, n, err, [&](uint32_t s) {
    const Crystal64 k = load64(cv, s);
    double t0, t1;
    if (!dintersect(k, 1.0, o, d, t0, t1)) return;
    if (!(t0 < g.step)) return;
    const double path = fmax(__dsub_rn(fmin(t1, g.step), t0), 0.0);
    if (!(path > 0.0)) return;
    if (pass) {
      if ((nh & 3) == 0) r = philox(g.photon, g.bounce, nh >> 2, TAG_HIT, k0, k1);
      const double u = ud(word(r, nh & 3));
      uint32_t cnt;
      E = absorb64(E, path, alpha, cv.sens64 ? cv.sens64[s] : static_cast<double>(cv.a[s].w), u, &cnt);
      if (cnt) atomicAdd(&counts[s], cnt);
      if (base + nh < id_cap) ids[base + nh] = s2id ? s2id[s] : s;
    }
    ++nh;
  });
  if (pass == 0) seg_count[i] = nh;
}

// Hits of arbitrary rays (whole ray, reference walk, exact geometry): over all crystals of the
// emulsion's tree, or over the developed ones (the scan's tree) with their expansion.
__global__ void k_replay_rays(const double* __restrict__ org, const double* __restrict__ dir, uint32_t nrays,
                              CrystalsView cv, RtView rv, const uint32_t* __restrict__ s2id, uint32_t n,
                              const double* exp64, int developed_only, int pass, uint32_t* ray_count,
                              const uint32_t* offsets, uint32_t* ids, uint32_t id_cap, double* chord_sum,
                              uint32_t* err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrays) return;
  const D3 o = d3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
  const D3 d = d3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
  const D3 inv = d3(__ddiv_rn(1.0, d.x), __ddiv_rn(1.0, d.y), __ddiv_rn(1.0, d.z));
  const uint32_t base = pass ? offsets[i] : 0u;
  uint32_t nh = 0;
  double L = 0.0;
  rt_crystals64(rv, o, inv, n, err, [&](uint32_t s) {
    const double e = developed_only ? exp64[s] : 1.0;
    const Crystal64 k = load64(cv, s);
    double t0, t1;
    if (!dintersect(k, e, o, d, t0, t1)) return;
    if (pass) {
      L = __dadd_rn(L, fmax(__dsub_rn(t1, t0), 0.0));
      if (base + nh < id_cap) ids[base + nh] = s2id ? s2id[s] : s;
    }
    ++nh;
  });
  if (pass == 0) {
    ray_count[i] = nh;
  } else if (chord_sum) {
    chord_sum[i] = L;
  }
}

// ---------------------------------------------------------------------------------------------
// Crystal records in a tree's element order: out[p] = in[ridx[p]] for p < n, so that the crystals
// of a leaf lie next to each other (TileDesc).
__global__ void k_element_records(const uint32_t* __restrict__ ridx, uint32_t n, const float4* __restrict__ a,
                                  const float4* __restrict__ q, const float4* __restrict__ d, float4* oa,
                                  float4* oq, float4* od, uint32_t* err) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t s = ridx[p];
  if (!index_ok(s < n, err, SITE_LEAF, s, n)) return;
  oa[p] = a[s];
  oq[p] = q[s];
  od[p] = d[s];
}

// The transport descriptor of an emulsion; a, q, d are its crystal records in the tree's element
// order (records, 3 n float4 written here).
TileDesc make_tile_desc(const fg_emulsion* em, const float* tile_dev, uint32_t tw, uint32_t th,
                        const fg_exposure_cfg& cfg, uint64_t seed, uint32_t* counts, float4* records,
                        uint32_t* err, cudaStream_t st) {
  TileDesc t{};
  float4* oa = records;
  float4* oq = records + em->n;
  float4* od = records + 2ull * em->n;
  if (em->n) {
    k_element_records<<<grid_for(em->n, 256), 256, 0, st>>>(em->rt.ridx.p, em->n, em->a.p, em->q.p, em->d.p, oa, oq,
                                                             od, err);
    FG_CUDA(cudaGetLastError());
  }
  t.a = oa;
  t.q = oq;
  t.d = od;
  t.rnode = em->rt.rnode.p;
  t.rleaf = em->rt.rleaf.p;
  t.ridx = em->rt.ridx.p;
  t.nnodes = static_cast<uint32_t>(em->rt.N);
  t.nrec = static_cast<uint32_t>(em->rt.R);
  t.reach = rt_reach(em->any_cubic ? em->max_half_dim : 0.0);
  t.s2id = em->sorted_to_id.p;
  t.n = em->n;
  t.counts = counts;
  t.tile = tile_dev;
  t.tw = tw;
  t.th = th;
  t.stride = tw;
  t.W = (float)em->cfg.width;
  t.H = (float)em->cfg.height;
  t.D = (float)em->cfg.depth;
  const double P = std::round(em->cfg.width * em->cfg.height * cfg.photons_per_sq_um);
  t.P = P > 0 ? static_cast<uint32_t>(P) : 0u;
  t.k0 = static_cast<uint32_t>(seed);
  t.k1 = static_cast<uint32_t>(seed >> 32);
  const fg_optics& o = em->cfg.optics;
  const double mu_t = o.absorption_coeff + o.scattering_coeff;
  t.mu_t = (float)mu_t;
  t.albedo = (float)(mu_t > 0.0 ? o.scattering_coeff / mu_t : 0.0);
  t.g = (float)o.anisotropy_g;
  const double r = (1.0 - o.refractive_index) / (1.0 + o.refractive_index);
  t.r0 = (float)(r * r);
  t.eff_r = (float)(o.antihalation_reflectance * std::pow(10.0, -2.0 * o.antihalation_density));
  t.theta_max = (float)cfg.illumination_angle_rad;
  t.alpha = (float)cfg.crystal_absorption_coeff;
  t.max_bounces = cfg.max_bounces;
  return t;
}

void launch_transport_shape(const TileDesc* tiles_dev, int ntiles, unsigned long long total,
                            const uint32_t* order, unsigned long long* counter, uint32_t* err,
                            unsigned long long* stats, unsigned blocks, unsigned threads, cudaStream_t st) {
  if (total == 0) return;
  FG_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st));
  const unsigned long long warps = (total + 31) / 32;
  const unsigned long long need = (warps * 32 + threads - 1) / threads;
  blocks = static_cast<unsigned>(std::max<unsigned long long>(std::min<unsigned long long>(blocks, need), 1));
  k_transport<<<blocks, threads, 0, st>>>(tiles_dev, ntiles, total, order, counter, err, stats);
  FG_CUDA(cudaGetLastError());
}

void expose(fg_engine* e, fg_emulsion* em, const float* tile_dev, uint32_t tw, uint32_t th,
            const fg_exposure_cfg& cfg, uint64_t seed, unsigned long long* photons_out) {
  cudaStream_t st = e->stream;
  DBuf<float4> records(3ull * std::max<uint32_t>(em->n, 1), st);
  TileDesc t = make_tile_desc(em, tile_dev, tw, th, cfg, seed, em->counts.p, records.p, e->d_err, st);
  if (photons_out) *photons_out = t.P;
  if (t.P == 0 || em->n == 0) return;
  DBuf<TileDesc> td(1, st);
  DBuf<unsigned long long> ctr(1, st);
  FG_CUDA(cudaMemcpyAsync(td.p, &t, sizeof(TileDesc), cudaMemcpyHostToDevice, st));
  launch_transport_shape(td.p, 1, t.P, nullptr, ctr.p, e->d_err, e->d_stats,
                         static_cast<unsigned>(e->sm_count) * 4, 256, st);
}

void replay_segments(fg_engine* e, fg_emulsion* em, const fg_exposure_cfg& cfg, uint64_t seed,
                     const fg_segment* segs_host, size_t nseg, uint32_t* offsets_host,
                     uint32_t* ids_host, size_t id_cap, size_t* nhits) {
  cudaStream_t st = e->stream;
  FG_REQUIRE(nseg < 0x7fffffffu, "too many segments");
  DBuf<fg_segment> segs(std::max<size_t>(nseg, 1), st);
  DBuf<uint32_t> cnt(nseg + 1, st), off(nseg + 1, st);
  if (nseg) FG_CUDA(cudaMemcpyAsync(segs.p, segs_host, nseg * sizeof(fg_segment), cudaMemcpyHostToDevice, st));
  const uint32_t k0 = static_cast<uint32_t>(seed), k1 = static_cast<uint32_t>(seed >> 32);
  const unsigned grid = grid_for(std::max<size_t>(nseg, 1), 128);
  const RtView rv = rt_view(em->rt);
  k_replay_segments<<<grid, 128, 0, st>>>(segs.p, (uint32_t)nseg, em->view(), rv, em->sorted_to_id.p, em->n,
                                          cfg.crystal_absorption_coeff, k0, k1, 0, cnt.p, nullptr, nullptr, 0,
                                          em->counts.p, e->d_err);
  FG_CUDA(cudaGetLastError());
  std::vector<uint32_t> hc(nseg + 1, 0);
  if (nseg) FG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, nseg * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  std::vector<uint32_t> ho(nseg + 1, 0);
  uint64_t acc = 0;
  for (size_t i = 0; i < nseg; ++i) {
    ho[i] = static_cast<uint32_t>(acc);
    acc += hc[i];
  }
  ho[nseg] = static_cast<uint32_t>(acc);
  FG_REQUIRE(acc < 0xffffffffull, "too many hits");
  if (nhits) *nhits = acc;
  FG_CUDA(cudaMemcpyAsync(off.p, ho.data(), (nseg + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  DBuf<uint32_t> ids(std::max<uint64_t>(std::min<uint64_t>(acc, id_cap), 1), st);
  k_replay_segments<<<grid, 128, 0, st>>>(segs.p, (uint32_t)nseg, em->view(), rv, em->sorted_to_id.p, em->n,
                                          cfg.crystal_absorption_coeff, k0, k1, 1, nullptr, off.p, ids.p,
                                          static_cast<uint32_t>(std::min<uint64_t>(acc, id_cap)), em->counts.p,
                                          e->d_err);
  FG_CUDA(cudaGetLastError());
  if (ids_host && acc) {
    FG_CUDA(cudaMemcpyAsync(ids_host, ids.p, std::min<uint64_t>(acc, id_cap) * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, st));
  }
  FG_CUDA(cudaStreamSynchronize(st));
  if (offsets_host) std::copy(ho.begin(), ho.end(), offsets_host);
}

void replay_rays(fg_engine* e, const fg_emulsion* em, const double* org_host,
                 const double* dir_host, size_t nrays, int developed_only, uint32_t* offsets_host,
                 uint32_t* ids_host, size_t id_cap, size_t* nhits, double* chord_host) {
  cudaStream_t st = e->stream;
  FG_REQUIRE(nrays < 0x7fffffffu, "too many rays");
  DBuf<double> org(std::max<size_t>(3 * nrays, 1), st), dir(std::max<size_t>(3 * nrays, 1), st);
  DBuf<uint32_t> cnt(nrays + 1, st), off(nrays + 1, st);
  DBuf<double> chord(std::max<size_t>(nrays, 1), st);
  if (nrays) {
    FG_CUDA(cudaMemcpyAsync(org.p, org_host, 3 * nrays * sizeof(double), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(dir.p, dir_host, 3 * nrays * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // Developed crystals are tested with their expansion over the scan's tree (developed crystals
  // only, transmittance.rs:86-89).
  RTreeBufs dev_tree;
  DBuf<uint32_t> dev_list;
  if (developed_only && em->n > 0) build_emulsion_tree(e, em, true, dev_tree, dev_list);
  const RtView rv = rt_view(developed_only ? dev_tree : em->rt);
  const unsigned grid = grid_for(std::max<size_t>(nrays, 1), 128);
  k_replay_rays<<<grid, 128, 0, st>>>(org.p, dir.p, (uint32_t)nrays, em->view(), rv, em->sorted_to_id.p, em->n,
                                      em->exp64.p, developed_only, 0, cnt.p, nullptr, nullptr, 0, nullptr, e->d_err);
  FG_CUDA(cudaGetLastError());
  std::vector<uint32_t> hc(nrays + 1, 0);
  if (nrays) FG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, nrays * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  std::vector<uint32_t> ho(nrays + 1, 0);
  uint64_t acc = 0;
  for (size_t i = 0; i < nrays; ++i) {
    ho[i] = static_cast<uint32_t>(acc);
    acc += hc[i];
  }
  ho[nrays] = static_cast<uint32_t>(acc);
  FG_REQUIRE(acc < 0xffffffffull, "too many hits");
  if (nhits) *nhits = acc;
  FG_CUDA(cudaMemcpyAsync(off.p, ho.data(), (nrays + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  DBuf<uint32_t> ids(std::max<uint64_t>(std::min<uint64_t>(acc, id_cap), 1), st);
  k_replay_rays<<<grid, 128, 0, st>>>(org.p, dir.p, (uint32_t)nrays, em->view(), rv, em->sorted_to_id.p, em->n,
                                      em->exp64.p, developed_only, 1, nullptr, off.p, ids.p,
                                      static_cast<uint32_t>(std::min<uint64_t>(acc, id_cap)), chord.p, e->d_err);
  FG_CUDA(cudaGetLastError());
  if (ids_host && acc)
    FG_CUDA(cudaMemcpyAsync(ids_host, ids.p, std::min<uint64_t>(acc, id_cap) * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, st));
  if (chord_host && nrays)
    FG_CUDA(cudaMemcpyAsync(chord_host, chord.p, nrays * sizeof(double), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  if (offsets_host) std::copy(ho.begin(), ho.end(), offsets_host);
}

}  // namespace fg
