// Batched tile pipeline: many exposure tiles (uneven sizes, stocks, push, seeds) rendered to
// negative density in one sequence of launches:
//   synthesis (column Bridson, 4 colour classes) -> thinning -> compaction in brick order -> the
//   reference tree (fg_rtree.cuh) -> persistent transport over all tiles' photons -> development ->
//   the reference tree over the developed crystals -> bins -> binned scan.
// Every kernel covers all tiles at once (per-tile descriptors in HBM, tile found by binary search
// on a prefix of work items), every buffer is allocated when the plan is made, and nothing waits
// on the host, so the sequence is captured once into a CUDA graph and replayed.  An autotuner
// picks the transport launch shape and the scan bin edge when the plan is made.
//
// The plain per-tile path (fg_render_tile, the drop-in for GpuEngine::render_tile_all_gpu,
// gpu.rs:491-938) is the same plan for one tile, made, run and freed per call.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "fg_internal.h"
#include "fg_scan.cuh"
#include "fg_synth.cuh"
#include "fg_transport.cuh"

namespace fg {

void launch_bridson(const SynthTile* tiles, int ntiles, const unsigned cols[4], int gdmax, uint32_t* cells,
                    uint32_t* npts, uint32_t* done, uint32_t* err, cudaStream_t st, uint32_t wait_limit = 0,
                    const uint32_t* probe = nullptr);
size_t bridson_smem(int gdmax);
void launch_synth_post(const SynthTile* tiles, int ntiles, unsigned long long max_cells, unsigned long long max_slots,
                       uint32_t* cells, uint32_t* npts, uint32_t* flags, cudaStream_t st);
void launch_emit(const SynthTile* tiles, int ntiles, unsigned long long max_slots, const uint32_t* cells,
                 const uint32_t* scan, float4* A, float4* Q, float4* D, uint64_t* keys, uint32_t* err,
                 cudaStream_t st);
void launch_transport_shape(const TileDesc* tiles_dev, int ntiles, unsigned long long total,
                            const uint32_t* order, unsigned long long* counter, uint32_t* err,
                            unsigned long long* stats, unsigned blocks, unsigned threads, cudaStream_t st);
void launch_photon_sort(const TileDesc* tiles_dev, int ntiles, unsigned long long total, unsigned long long ncells,
                        uint32_t* cnt, const uint32_t* off, uint32_t* cur, uint32_t* order, uint32_t* err,
                        cudaStream_t st);
void launch_density(float* d, unsigned long long n, cudaStream_t st);
void launch_scan(const ScanTile* tiles, int ntiles, unsigned long long nbins, unsigned threads, uint32_t* err,
                 unsigned long long* stats, cudaStream_t st);
void launch_scan_prep(const ScanTile* tiles, int ntiles, unsigned long long nslots, ScanPrep* prep,
                      cudaStream_t st);
void launch_scan_prep_list(const ScanTile* tiles, int ntiles, const uint32_t* list, const uint32_t* nlist,
                           unsigned long long cap, ScanPrep* prep, cudaStream_t st);
uint32_t scan_bin_px(uint32_t spp);

// Nodes per crystal slot of the tile trees: the reference tree has about 0.67 nodes per crystal and
// a tile holds about 0.72 crystals per slot, so 0.8 leaves a wide margin (an overflow fails the run).
constexpr double RT_NODE_FRAC = 0.8;

// Per-tile state for the batched trees, development and binning kernels.
struct __align__(16) BTile {
  unsigned long long cbase;   // first crystal slot (also the tile's first element of its trees)
  unsigned long long nbase;   // first node of the tile's trees
  unsigned long long bin_base;
  double fe, prox;            // filament expansion, clumping proximity (development.rs:12-27)
  double max_base;            // largest undeveloped max_dim (device-written)
  uint32_t n;                 // crystals (device-written)
  uint32_t thr;               // threshold photons
  uint32_t nbx, nby;
  float binw_x, binw_y;
  float pad;                  // leaf box padding
  uint32_t ncap;              // node capacity of the tile's trees
  uint32_t rbase, rcap;       // first walk record of the tile's tree, and their count
};

__device__ __forceinline__ int btile_of(const BTile* tiles, int ntiles, unsigned long long g) {
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].cbase <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void k_set_n(const SynthTile* syn, int ntiles, const uint32_t* slot_scan, BTile* bt, TileDesc* td,
                        ScanTile* sc, uint32_t* ncrys, RTile* rt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint32_t n = slot_scan[syn[t].slot_base + (1ull << (2 * syn[t].slot_bits))] - slot_scan[syn[t].slot_base];
  const uint32_t nn = min(n, syn[t].ccap);
  bt[t].n = nn;
  bt[t].max_base = 0.0;
  td[t].n = nn;
  sc[t].n = nn;
  ncrys[t] = nn;
  rt[t].n = nn;
}

// Inputs of the scan's tree per tile: the tile's developed crystals in slot order (transmittance.rs:
// 86-89 keeps them in crystal order), from the exclusive sum of the developed flags.
__global__ void k_scan_tree_tiles(const BTile* bt, int ntiles, const uint32_t* devscan, const uint32_t* devlist,
                                  RTile* rt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const uint32_t first = devscan[bt[t].cbase], last = devscan[bt[t].cbase + bt[t].n];
  rt[t].order = devlist + first;
  rt[t].obase = bt[t].cbase;
  rt[t].n = last - first;
}

// Crystal records of every tile in its tree's element order (TileDesc): position p of tile t holds
// the crystal ridx[p] of that tile, so a leaf's crystals lie next to each other.
__global__ void k_element_records_b(const BTile* __restrict__ bt, int ntiles, unsigned long long ncap,
                                    const uint32_t* __restrict__ ridx, const float4* __restrict__ A,
                                    const float4* __restrict__ Q, const float4* __restrict__ D, float4* EA,
                                    float4* EQ, float4* ED, uint32_t* err) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= ncap) return;
  const BTile& t = bt[btile_of(bt, ntiles, g)];
  const unsigned long long p = g - t.cbase;
  if (p >= t.n) return;
  const uint32_t s = ridx[g];
  if (!index_ok(s < t.n, err, SITE_LEAF, s, t.n)) return;
  EA[g] = A[t.cbase + s];
  EQ[g] = Q[t.cbase + s];
  ED[g] = D[t.cbase + s];
}

// ---- development (development.rs:59-188), batched; see fg_develop.cu for the reasoning ----

// Largest max_dim of each tile's crystals (the reach of the development's proximity search):
// blockIdx.y is the tile, its blocks stride over the tile's crystals; a warp maximum, then one
// atomic per warp (positive doubles order as their bit patterns).
__global__ void k_maxdim_b(BTile* bt, const float4* __restrict__ D) {
  BTile& T = bt[blockIdx.y];
  const uint32_t n = T.n;
  float m = 0.0f;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 d = D[T.cbase + i];
    m = fmaxf(m, fmaxf(fmaxf(d.x, d.y), d.z));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f)
    atomicMax(reinterpret_cast<unsigned long long*>(&T.max_base),
              static_cast<unsigned long long>(__double_as_longlong(static_cast<double>(m))));
}

__global__ void k_threshold_b(const BTile* __restrict__ bt, int ntiles, unsigned long long ncap,
                              const uint32_t* counts, uint8_t* developed, int* parent, uint32_t* devflag) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= ncap) return;
  const BTile& t = bt[btile_of(bt, ntiles, g)];
  const bool in = g - t.cbase < t.n;
  const bool dv = in && counts[g] >= t.thr;
  developed[g] = dv ? 1 : 0;
  devflag[g] = dv ? 1u : 0u;
  parent[g] = static_cast<int>(g);
}

// Developed slots in slot order (from the exclusive scan of the flags), so that the touch queries
// run in full, spatially coherent warps.
__global__ void k_devlist_b(unsigned long long ncap, const uint32_t* __restrict__ devflag,
                            const uint32_t* __restrict__ devscan, uint32_t* __restrict__ list) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= ncap || !devflag[g]) return;
  list[devscan[g]] = static_cast<uint32_t>(g);
}

__device__ __forceinline__ int uf_find_b(int* parent, int x, uint32_t* err) {
  for (int it = 0; it < (1 << 22); ++it) {
    const int p = __ldcg(&parent[x]);
    if (p == x) return x;
    const int gp = __ldcg(&parent[p]);
    if (gp != p) atomicCAS(&parent[x], p, gp);
    x = gp;
  }
  atomicOr(err, ERR_SPIN_LIMIT);
  return x;
}

__device__ __forceinline__ void uf_unite_b(int* parent, int a, int b, uint32_t* err) {
  for (int it = 0; it < (1 << 20); ++it) {
    a = uf_find_b(parent, a, err);
    b = uf_find_b(parent, b, err);
    if (a == b) return;
    if (a > b) { const int tmp = a; a = b; b = tmp; }
    const int old = atomicCAS(&parent[b], b, a);
    if (old == b) return;
    b = old;
  }
  atomicOr(err, ERR_SPIN_LIMIT);
}

// Links each developed crystal to the developed crystals it touches (union-find), walking the
// tile's reference tree with the query box: a leaf is reached iff its box and its ancestors' boxes
// overlap the query (ancestor boxes contain their descendants'), and a crystal within the touch
// distance lies inside its own leaf box, so the query finds it whatever the tree (bvh.rs:350-402);
// the union-find roots do not depend on the order of the unions.
__global__ void k_link_b(const BTile* __restrict__ bt, int ntiles, unsigned long long ncap,
                         const float4* __restrict__ A, const float4* __restrict__ D, const Node4* __restrict__ rnode_all,
                         const uint2* __restrict__ rleaf_all, const uint32_t* __restrict__ ridx_all,
                         const uint8_t* __restrict__ developed, int* parent, const uint32_t* __restrict__ list,
                         const uint32_t* __restrict__ ndev, uint32_t* err) {
  const unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (i >= ncap || i >= *ndev) return;
  const unsigned long long g = list[i];
  const BTile& t = bt[btile_of(bt, ntiles, g)];
  const uint32_t s = static_cast<uint32_t>(g - t.cbase);
  const Node4* nodes = rnode_all + t.rbase;
  const uint2* leaves = rleaf_all + t.nbase;
  const uint32_t* ridx = ridx_all + t.cbase;
  const float4* Ab = A + t.cbase;
  const float4* Db = D + t.cbase;
  const uint8_t* dev = developed + t.cbase;
  const float4 a = Ab[s], d = Db[s];
  // Synthesized crystals are exactly their FP32 values, so the reference's FP64 expressions can
  // be evaluated from them directly when the FP32 margin is too thin.
  const double rc = __dmul_rn(static_cast<double>(fmaxf(fmaxf(d.x, d.y), d.z)), t.fe);
  const double search = __dmul_rn(__dadd_rn(rc, __dmul_rn(t.max_base, t.fe)), t.prox);
  const float R = static_cast<float>(search) * 1.0001f + 1e-3f;
  const float3 lo = make_float3(a.x - R, a.y - R, a.z - R), hi = make_float3(a.x + R, a.y + R, a.z + R);
  const float fef = static_cast<float>(t.fe), proxf = static_cast<float>(t.prox);
  const float rcf = fmaxf(fmaxf(d.x, d.y), d.z) * fef;
  if (t.n < 2) return;
  const uint32_t nmax = t.ncap;
  auto test = [&](uint32_t j) {
    if (j <= s || j >= t.n || !dev[j]) return;
    const float4 aj = Ab[j], dj = Db[j];
    const float dx = aj.x - a.x, dy = aj.y - a.y, dz = aj.z - a.z;
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float touch = (rcf + fmaxf(fmaxf(dj.x, dj.y), dj.z) * fef) * proxf;
    const float t2 = touch * touch;
    const float margin = 1e-5f * t2 + 1e-6f;
    bool hit;
    if (d2 < t2 - margin) {
      hit = true;
    } else if (d2 > t2 + margin) {
      hit = false;
    } else {
      const double rn = __dmul_rn(static_cast<double>(fmaxf(fmaxf(dj.x, dj.y), dj.z)), t.fe);
      const double tt = __dmul_rn(__dadd_rn(rc, rn), t.prox);
      const double ex = __dsub_rn(static_cast<double>(aj.x), static_cast<double>(a.x));
      const double ey = __dsub_rn(static_cast<double>(aj.y), static_cast<double>(a.y));
      const double ez = __dsub_rn(static_cast<double>(aj.z), static_cast<double>(a.z));
      hit = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez)) <= __dmul_rn(tt, tt);
    }
    if (hit) uf_unite_b(parent, static_cast<int>(g), static_cast<int>(t.cbase + j), err);
  };
  auto leaf = [&](uint32_t id) {
    if (!index_ok(id < nmax, err, SITE_LEAF, id, nmax)) return;
    const uint2 L = leaves[id];
    if (!index_ok(L.x + L.y <= t.n, err, SITE_LEAF, L.x, L.y)) return;
    for (uint32_t k = 0; k < L.y; ++k) test(ridx[L.x + k]);
  };
  rt_walk4_box(nodes, lo, hi, t.rcap, err, leaf);
}

__global__ void k_roots_b(unsigned long long ncap, const uint8_t* developed, int* parent, uint32_t* size,
                          uint32_t* err) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= ncap || !developed[g]) return;
  const int r = uf_find_b(parent, static_cast<int>(g), err);
  parent[g] = r;
  atomicAdd(&size[r], 1u);
}

// Also counts the clumps (development.rs:107-108: one per connected component of developed
// crystals, singletons included), one warp-aggregated add per warp.
__global__ void k_finalize_b(const BTile* __restrict__ bt, int ntiles, unsigned long long ncap,
                             const uint8_t* developed, const int* parent, const uint32_t* size, double* exp64,
                             unsigned long long* clumps) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  bool root = false;
  if (g < ncap) {
    if (!developed[g]) {
      exp64[g] = 0.0;
    } else {
      const BTile& t = bt[btile_of(bt, ntiles, g)];
      const int p = parent[g];
      const uint32_t sz = size[p];
      double e = t.fe;
      if (sz > 1)
        e = __dmul_rn(t.fe, __dadd_rn(1.15, __dmul_rn(0.18, static_cast<double>((sz < 6 ? sz : 6) - 1))));
      exp64[g] = e;
      root = p == static_cast<int>(g);
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, root);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(clumps, static_cast<unsigned long long>(__popc(m)));
}

// ---- scan bins (per tile grid of bin_px x bin_px pixels) ----

__device__ __forceinline__ void bin_span(float l, float h, float binw, uint32_t nb, uint32_t& b0, uint32_t& b1) {
  const float lo = (l - 1e-3f) / binw, hi = (h + 1e-3f) / binw;
  b0 = static_cast<uint32_t>(fminf(fmaxf(floorf(lo), 0.0f), static_cast<float>(nb - 1)));
  b1 = static_cast<uint32_t>(fminf(fmaxf(floorf(hi), 0.0f), static_cast<float>(nb - 1)));
}

// A developed crystal goes to every bin its leaf box (in the scan's tree) overlaps.
__global__ void k_bin_b(const BTile* __restrict__ bt, int ntiles, unsigned long long ncap,
                        const uint8_t* __restrict__ developed, const double* __restrict__ box64,
                        const uint32_t* __restrict__ leafof, uint32_t* cnt, const uint32_t* off, uint32_t* cursor,
                        uint32_t* items, unsigned long long item_cap, uint32_t* err) {
  const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  if (g >= ncap || !developed[g]) return;
  const BTile& t = bt[btile_of(bt, ntiles, g)];
  const double* lb = box64 + 6ull * (t.nbase + leafof[g]);
  uint32_t x0, x1, y0, y1;
  bin_span(static_cast<float>(lb[0]), static_cast<float>(lb[3]), t.binw_x, t.nbx, x0, x1);
  bin_span(static_cast<float>(lb[1]), static_cast<float>(lb[4]), t.binw_y, t.nby, y0, y1);
  const uint32_t s = static_cast<uint32_t>(g - t.cbase);
  for (uint32_t by = y0; by <= y1; ++by)
    for (uint32_t bx = x0; bx <= x1; ++bx) {
      const unsigned long long b = t.bin_base + by * t.nbx + bx;
      if (!off) {
        atomicAdd(&cnt[b], 1u);
      } else {
        const unsigned long long k = off[b] + atomicAdd(&cursor[b], 1u);
        if (k < item_cap) items[k] = s; else atomicOr(err, ERR_LIST_OVERFLOW);
      }
    }
}

}  // namespace fg

using namespace fg;

// ---------------------------------------------------------------------------------------------
struct fg_batch {
  fg_engine* e = nullptr;
  uint32_t ntiles = 0;
  std::vector<fg_tile_params> params;
  std::vector<SynthTile> syn;
  std::vector<TileDesc> td;
  std::vector<ScanTile> sc;
  std::vector<BTile> bt;
  std::vector<unsigned long long> exp_off, out_off;
  DBuf<SynthTile> d_syn;
  DBuf<TileDesc> d_td;
  DBuf<ScanTile> d_sc;
  DBuf<BTile> d_bt;
  DBuf<uint32_t> cells, npts, flags, slot_scan, ncrys;  // flags: points per brick, slot_scan: their exclusive sum
  DBuf<uint32_t> coldone;  // one flag per synthesis column
  DBuf<uint32_t> probe;    // the failure drill's flag (zero, never set)
  uint32_t wait_limit = 0;
  bool wait_probe = false;
  unsigned long long maxcells = 0, maxslots = 0;  // the largest tile's cells and bricks
  DBuf<float4> A, Q, D;
  DBuf<float4> EA, EQ, ED;  // A, Q, D in the transport tree's element order (TileDesc)
  DBuf<uint64_t> keys;
  RTreeBufs rt;             // the reference tree of every tile: over its crystals, then its developed ones
  DBuf<RTile> rt_scan;      // the tree tiles of the scan's build (developed crystals, their expansion)
  DBuf<int> parent;
  DBuf<uint32_t> counts, size;
  DBuf<uint8_t> developed;
  DBuf<double> exp64;
  DBuf<ScanPrep> prep;  // staging terms of developed crystals for the scan
  DBuf<uint32_t> devflag, devscan, devlist;  // developed slots, compacted for the touch queries
  DBuf<uint32_t> bin_cnt, bin_off, bin_cur, bin_items;
  DBuf<uint32_t> pcnt, poff, pcur, porder;  // photon ordering by emission cell
  unsigned long long npcells = 0;
  DBuf<float> exposure, d_neg;
  DBuf<unsigned long long> counter;
  DBuf<unsigned long long> dstats;  // [0] transport hits, [1] scan FP64 fallbacks, [2] scan hits, [3] clumps
  DBuf<unsigned char> cub_tmp;
  size_t cub_bytes = 0;
  unsigned long long ncells = 0, nslots = 0, ncap = 0, nbins = 0, item_cap = 0, photons = 0, rays = 0;  // nslots: bricks
  unsigned long long exp_total = 0, out_total = 0;
  int gdmax = 0;
  unsigned cols[4] = {0, 0, 0, 0};
  unsigned tr_blocks = 0, tr_threads = 256, scan_threads = 256;
  uint32_t bin_px = 8;
  bool use_graph = true;
  bool tune_pending = false;  // autotune (and capture) at the first run, once exposure is set
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[9] = {};  // stage marks 0-5, the timing start 6, k_bridson's end 7 and start 8
  fg_batch_stats stats{};

  ~fg_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& x : ev)
      if (x) cudaEventDestroy(x);
  }
};

namespace fg {

static void derive_tile(const fg_tile_params& p, SynthTile& s, TileDesc& t, ScanTile& c, BTile& b) {
  FG_REQUIRE(p.film_w > 0 && p.film_h > 0 && p.film_d > 0, "film dimensions must be positive");
  FG_REQUIRE(p.width_px > 0 && p.height_px > 0, "tile size must be positive");
  FG_REQUIRE(p.r_min > 0, "r_min must be positive");
  FG_REQUIRE(p.morphology >= 0 && p.morphology <= 2, "morphology out of range");
  const double W = p.film_w, H = p.film_h, Dd = p.film_d, r = p.r_min;
  const double cell = r / std::sqrt(3.0);
  s = SynthTile{};
  s.cell = static_cast<float>(cell);
  s.gw = static_cast<uint32_t>(std::ceil(W / cell));
  s.gh = static_cast<uint32_t>(std::ceil(H / cell));
  s.gd = static_cast<uint32_t>(std::ceil(Dd / cell));
  FG_REQUIRE(s.gw <= 16000 && s.gh <= 16000 && s.gd <= 100, "tile too large for the synthesis grid");
  FG_REQUIRE(static_cast<unsigned long long>(s.gw) * s.gh * s.gd < (1ull << 31), "tile too large for the synthesis grid");
  s.nbx = (s.gw + SYN_B - 1) / SYN_B;
  s.nby = (s.gh + SYN_B - 1) / SYN_B;
  s.XW = static_cast<uint32_t>(std::ceil(W * SYN_Q / cell));
  s.YW = static_cast<uint32_t>(std::ceil(H * SYN_Q / cell));
  s.ZW = static_cast<uint32_t>(std::ceil(Dd * SYN_Q / cell));
  uint32_t bits = 0, zb = 0;
  while ((1u << bits) < std::max(s.gw, s.gh)) ++bits;
  while ((1u << zb) < s.gd) ++zb;
  s.brick_bits = zb;
  s.slot_bits = bits > zb ? bits - zb : 0;
  const unsigned long long slots = (1ull << (2 * s.slot_bits)) << (3 * zb);
  FG_REQUIRE(slots < (1ull << 31), "tile too large for the synthesis grid");
  s.slots = static_cast<uint32_t>(slots);
  const double vol = W * H * Dd;
  const double cap = std::min(0.8 * vol / (r * r * r) + 64.0, static_cast<double>(s.gw) * s.gh * s.gd);
  s.ccap = static_cast<uint32_t>(cap);
  s.target = static_cast<uint32_t>(std::llround(bridson_density(W, H, Dd, r) * vol));
  s.k0 = static_cast<uint32_t>(p.seed);
  s.k1 = static_cast<uint32_t>(p.seed >> 32);
  double mu = std::log(p.mean_crystal_radius), sg = p.size_variance;
  if (!(sg >= 0.0) || !std::isfinite(mu) || !std::isfinite(sg)) {  // LogNormal::new fallback
    mu = 0.0;
    sg = 0.2;
  }
  s.mu = static_cast<float>(mu);
  s.sg = static_cast<float>(sg);
  s.rmax = static_cast<float>(r * 0.48);
  s.base_sens = static_cast<float>(p.base_sensitivity);
  s.aspect = static_cast<float>(p.tabular_aspect_ratio);
  s.morph = p.morphology;
  // Transport (seed + 1) and scan (seed + 2) as the tile worker derives them.
  t = TileDesc{};
  t.tw = p.width_px;
  t.th = p.height_px;
  t.stride = p.width_px;
  t.W = static_cast<float>(W);
  t.H = static_cast<float>(H);
  t.D = static_cast<float>(Dd);
  const double pps = p.photons_per_sq_um * std::max(p.exposure, 0.05);
  const double P = std::round(W * H * pps);
  FG_REQUIRE(P < 4e9, "too many photons in one tile");
  t.P = P > 0 ? static_cast<uint32_t>(P) : 0u;
  const uint64_t es = p.seed + 1, ss = p.seed + 2;
  t.k0 = static_cast<uint32_t>(es);
  t.k1 = static_cast<uint32_t>(es >> 32);
  const fg_optics& o = p.optics;
  const double mu_t = o.absorption_coeff + o.scattering_coeff;
  t.mu_t = static_cast<float>(mu_t);
  t.albedo = static_cast<float>(mu_t > 0 ? o.scattering_coeff / mu_t : 0.0);
  t.g = static_cast<float>(o.anisotropy_g);
  const double rr = (1.0 - o.refractive_index) / (1.0 + o.refractive_index);
  t.r0 = static_cast<float>(rr * rr);
  t.eff_r = static_cast<float>(o.antihalation_reflectance * std::pow(10.0, -2.0 * o.antihalation_density));
  t.theta_max = static_cast<float>(p.illumination_angle_rad);
  t.alpha = static_cast<float>(p.crystal_absorption_coeff);
  t.max_bounces = p.max_bounces;
  c = ScanTile{};
  const uint32_t spp = std::max<uint32_t>(p.samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::lround(std::sqrt(static_cast<double>(spp))));
  c.g = g;
  c.spp = std::max<uint32_t>(g * g, 1);
  FG_REQUIRE(c.spp <= SCAN_THREADS, "samples_per_pixel too large");
  c.w = p.width_px;
  c.h = p.height_px;
  c.pw = W / p.width_px;
  c.ph = H / p.height_px;
  c.z0 = Dd + 0.1;
  c.seed = ss;
  c.sigma = static_cast<float>(p.silver_opacity);
  c.mode = 0;
  set_jitter_units(c);
  b = BTile{};
  b.fe = p.filament_expansion;
  b.prox = p.clumping_proximity_factor;
  b.thr = p.threshold_photons;
  b.pad = static_cast<float>(std::max(std::max(W, H), Dd) * 2e-6 + 1e-5);
}

// Places the per-tile bins for a bin edge and refreshes the scan / bin descriptors.
static void layout_bins(fg_batch* B, uint32_t bin_px) {
  unsigned long long base = 0;
  for (uint32_t i = 0; i < B->ntiles; ++i) {
    ScanTile& c = B->sc[i];
    BTile& b = B->bt[i];
    const uint32_t bp = std::min<uint32_t>(bin_px, scan_bin_px(c.spp));
    c.bin_px = bp;
    c.nbx = (c.w + bp - 1) / bp;
    c.nby = (c.h + bp - 1) / bp;
    c.bin_base = base;
    b.bin_base = base;
    b.nbx = c.nbx;
    b.nby = c.nby;
    b.binw_x = static_cast<float>(bp * c.pw);
    b.binw_y = static_cast<float>(bp * c.ph);
    base += static_cast<unsigned long long>(c.nbx) * c.nby;
  }
  B->nbins = base;
  unsigned mx = 32;
  for (uint32_t i = 0; i < B->ntiles; ++i)
    mx = std::max(mx, ((B->sc[i].bin_px * B->sc[i].bin_px * B->sc[i].spp + 31) / 32) * 32);
  B->scan_threads = mx;
  B->bin_px = bin_px;
}

static void upload_descriptors(fg_batch* B, cudaStream_t st) {
  // Device pointers inside the descriptors depend on the buffers.  The per-tile crystal counts n
  // are device-written (k_set_n from the compaction scan); the host copies hold 0, so they are
  // re-derived on the device right after the copy.
  for (uint32_t i = 0; i < B->ntiles; ++i) {
    const unsigned long long cb = B->syn[i].cbase;
    TileDesc& t = B->td[i];
    t.a = B->EA.p + cb;
    t.q = B->EQ.p + cb;
    t.d = B->ED.p + cb;
    const unsigned long long nb = B->bt[i].nbase;
    t.rnode = B->rt.rnode.p + B->bt[i].rbase;
    t.rleaf = B->rt.rleaf.p + nb;
    t.ridx = B->rt.ridx.p + cb;
    t.s2id = nullptr;
    t.counts = B->counts.p + cb;
    t.tile = B->exposure.p + B->exp_off[i];
    ScanTile& c = B->sc[i];
    c.prep = B->prep.p + cb;
    c.slot_base = cb;
    c.a = B->A.p + cb;
    c.q = B->Q.p + cb;
    c.d = B->D.p + cb;
    c.pos64 = c.dims64 = c.quat64 = nullptr;
    c.developed = B->developed.p + cb;
    c.exp64 = B->exp64.p + cb;
    c.lbox64 = B->rt.box64.p + 6 * nb;
    c.leafof = B->rt.leafof.p + cb;
    c.sigma_c = nullptr;
    c.bin_off = B->bin_off.p + c.bin_base;
    c.bin_items = B->bin_items.p;
    c.items_cap = static_cast<uint32_t>(std::min<unsigned long long>(B->item_cap, 0xffffffffull));
    c.out = nullptr;
    c.image8 = nullptr;
    c.d_neg = B->d_neg.p + B->out_off[i];
    c.ray_hits = nullptr;
    B->bt[i].cbase = cb;
  }
  FG_CUDA(cudaMemcpyAsync(B->d_syn.p, B->syn.data(), B->ntiles * sizeof(SynthTile), cudaMemcpyHostToDevice, st));
  FG_CUDA(cudaMemcpyAsync(B->d_td.p, B->td.data(), B->ntiles * sizeof(TileDesc), cudaMemcpyHostToDevice, st));
  FG_CUDA(cudaMemcpyAsync(B->d_sc.p, B->sc.data(), B->ntiles * sizeof(ScanTile), cudaMemcpyHostToDevice, st));
  FG_CUDA(cudaMemcpyAsync(B->d_bt.p, B->bt.data(), B->ntiles * sizeof(BTile), cudaMemcpyHostToDevice, st));
  k_set_n<<<grid_for(B->ntiles, 128), 128, 0, st>>>(B->d_syn.p, static_cast<int>(B->ntiles), B->slot_scan.p, B->d_bt.p,
                                                    B->d_td.p, B->d_sc.p, B->ncrys.p, B->rt.tiles.p);
  FG_CUDA(cudaGetLastError());
}

static void cub_scan(fg_batch* B, const uint32_t* in, uint32_t* out, unsigned long long n, cudaStream_t st) {
  size_t bytes = B->cub_bytes;
  FG_CUDA(cub::DeviceScan::ExclusiveSum(B->cub_tmp.p, bytes, in, out, static_cast<int64_t>(n), st));
}

// Stages; each only enqueues work on `st`.
static void mark(cudaEvent_t ev, cudaStream_t st, bool capturing);

static void stage_synth(fg_batch* B, cudaStream_t st, bool capturing = false) {
  fg_engine* e = B->e;
  const int nt = static_cast<int>(B->ntiles);
  FG_CUDA(cudaMemsetAsync(B->dstats.p, 0, 4 * sizeof(unsigned long long), st));
  FG_CUDA(cudaMemsetAsync(B->cells.p, 0, B->ncells * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(B->npts.p, 0, B->ntiles * sizeof(uint32_t), st));
  mark(B->ev[8], st, capturing);
  launch_bridson(B->d_syn.p, nt, B->cols, B->gdmax, B->cells.p, B->npts.p, B->coldone.p, e->d_err, st,
                 B->wait_limit, B->wait_probe ? B->probe.p : nullptr);
  mark(B->ev[7], st, capturing);
  FG_CUDA(cudaMemsetAsync(B->flags.p + B->nslots, 0, sizeof(uint32_t), st));
  launch_synth_post(B->d_syn.p, nt, B->maxcells, B->maxslots, B->cells.p, B->npts.p, B->flags.p, st);
  cub_scan(B, B->flags.p, B->slot_scan.p, B->nslots + 1, st);
  launch_emit(B->d_syn.p, nt, B->maxslots, B->cells.p, B->slot_scan.p, B->A.p, B->Q.p, B->D.p, B->keys.p, e->d_err,
              st);
  k_set_n<<<grid_for(B->ntiles, 128), 128, 0, st>>>(B->d_syn.p, nt, B->slot_scan.p, B->d_bt.p, B->d_td.p, B->d_sc.p,
                                                    B->ncrys.p, B->rt.tiles.p);
  FG_CUDA(cudaGetLastError());
}

// The reference tree of every tile over its crystals (in slot order), for the transport and the
// development's touch queries.
static void stage_bvh(fg_batch* B, cudaStream_t st) {
  rtree_build(B->rt, B->e->d_err, st);
  k_element_records_b<<<grid_for(B->ncap, 256), 256, 0, st>>>(B->d_bt.p, static_cast<int>(B->ntiles), B->ncap,
                                                              B->rt.ridx.p, B->A.p, B->Q.p, B->D.p, B->EA.p,
                                                              B->EQ.p, B->ED.p, B->e->d_err);
  FG_CUDA(cudaGetLastError());
}

static void stage_transport(fg_batch* B, cudaStream_t st) {
  FG_CUDA(cudaMemsetAsync(B->counts.p, 0, B->ncap * sizeof(uint32_t), st));
  launch_transport_shape(B->d_td.p, static_cast<int>(B->ntiles), B->photons, B->porder.p, B->counter.p,
                         B->e->d_err, B->dstats.p, B->tr_blocks, B->tr_threads, st);
}

// Orders photon ids by emission cell (independent of the crystals: runs with synthesis).
static void stage_photon_order(fg_batch* B, cudaStream_t st) {
  const int nt = static_cast<int>(B->ntiles);
  FG_CUDA(cudaMemsetAsync(B->pcnt.p, 0, (B->npcells + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(B->pcur.p, 0, (B->npcells + 1) * sizeof(uint32_t), st));
  launch_photon_sort(B->d_td.p, nt, B->photons, B->npcells, B->pcnt.p, nullptr, nullptr, nullptr, B->e->d_err, st);
  cub_scan(B, B->pcnt.p, B->poff.p, B->npcells + 1, st);
  launch_photon_sort(B->d_td.p, nt, B->photons, B->npcells, nullptr, B->poff.p, B->pcur.p, B->porder.p, B->e->d_err,
                     st);
}

static void stage_develop(fg_batch* B, cudaStream_t st) {
  const int nt = static_cast<int>(B->ntiles);
  fg_engine* e = B->e;
  const unsigned G = grid_for(B->ncap, 256);
  {
    uint32_t cmax = 1;  // the largest tile's crystal capacity
    for (int i = 0; i < nt; ++i) cmax = std::max(cmax, B->syn[i].ccap);
    const unsigned bx = std::min(std::max((cmax + 2047u) / 2048u, 1u), 2048u);
    FG_REQUIRE(nt <= 65535, "too many tiles for one launch");
    k_maxdim_b<<<dim3(bx, static_cast<unsigned>(nt)), 256, 0, st>>>(B->d_bt.p, B->D.p);
  }
  k_threshold_b<<<G, 256, 0, st>>>(B->d_bt.p, nt, B->ncap, B->counts.p, B->developed.p, B->parent.p, B->devflag.p);
  FG_CUDA(cudaMemsetAsync(B->devflag.p + B->ncap, 0, sizeof(uint32_t), st));
  cub_scan(B, B->devflag.p, B->devscan.p, B->ncap + 1, st);
  k_devlist_b<<<G, 256, 0, st>>>(B->ncap, B->devflag.p, B->devscan.p, B->devlist.p);
  k_link_b<<<G, 256, 0, st>>>(B->d_bt.p, nt, B->ncap, B->A.p, B->D.p, B->rt.rnode.p, B->rt.rleaf.p, B->rt.ridx.p,
                              B->developed.p, B->parent.p, B->devlist.p, B->devscan.p + B->ncap, e->d_err);
  FG_CUDA(cudaMemsetAsync(B->size.p, 0, B->ncap * sizeof(uint32_t), st));
  k_roots_b<<<G, 256, 0, st>>>(B->ncap, B->developed.p, B->parent.p, B->size.p, e->d_err);
  k_finalize_b<<<G, 256, 0, st>>>(B->d_bt.p, nt, B->ncap, B->developed.p, B->parent.p, B->size.p, B->exp64.p,
                                  B->dstats.p + 3);
  FG_CUDA(cudaGetLastError());
}

static void stage_scan(fg_batch* B, cudaStream_t st) {
  const int nt = static_cast<int>(B->ntiles);
  fg_engine* e = B->e;
  const unsigned G = grid_for(B->ncap, 256);
  // The scan's tree: the same buffers, rebuilt over each tile's developed crystals (the transport
  // and the touch queries are done with the first tree by now).
  k_scan_tree_tiles<<<grid_for(B->ntiles, 128), 128, 0, st>>>(B->d_bt.p, nt, B->devscan.p, B->devlist.p, B->rt_scan.p);
  rtree_build(B->rt, e->d_err, st, B->rt_scan.p);
  launch_scan_prep_list(B->d_sc.p, nt, B->devlist.p, B->devscan.p + B->ncap, B->ncap, B->prep.p, st);
  FG_CUDA(cudaMemsetAsync(B->bin_cnt.p, 0, (B->nbins + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(B->bin_cur.p, 0, (B->nbins + 1) * sizeof(uint32_t), st));
  k_bin_b<<<G, 256, 0, st>>>(B->d_bt.p, nt, B->ncap, B->developed.p, B->rt.box64.p, B->rt.leafof.p, B->bin_cnt.p,
                             nullptr, nullptr, nullptr, 0, e->d_err);
  cub_scan(B, B->bin_cnt.p, B->bin_off.p, B->nbins + 1, st);
  k_bin_b<<<G, 256, 0, st>>>(B->d_bt.p, nt, B->ncap, B->developed.p, B->rt.box64.p, B->rt.leafof.p, nullptr,
                             B->bin_off.p, B->bin_cur.p, B->bin_items.p, B->item_cap, e->d_err);
  FG_CUDA(cudaGetLastError());
  launch_scan(B->d_sc.p, nt, B->nbins, B->scan_threads, e->d_err, B->dstats.p, st);
  launch_density(B->d_neg.p, B->out_total, st);
}

// Stage events: inside a graph capture they must be external records so that every replay
// records them again (a plain record would become an internal dependency only).
static void mark(cudaEvent_t ev, cudaStream_t st, bool capturing) {
  FG_CUDA(cudaEventRecordWithFlags(ev, st, capturing ? cudaEventRecordExternal : cudaEventRecordDefault));
}

static void enqueue_all(fg_batch* B, cudaStream_t st, bool capturing = false) {
  mark(B->ev[0], st, capturing);
  stage_synth(B, st, capturing);
  stage_photon_order(B, st);
  mark(B->ev[1], st, capturing);
  stage_bvh(B, st);
  mark(B->ev[2], st, capturing);
  stage_transport(B, st);
  mark(B->ev[3], st, capturing);
  stage_develop(B, st);
  mark(B->ev[4], st, capturing);
  stage_scan(B, st);
  mark(B->ev[5], st, capturing);
}

static float ev_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  FG_CUDA(cudaEventElapsedTime(&ms, a, b));
  return ms;
}

// Picks the transport launch shape and the scan bin edge by timing candidates on this batch.
static void autotune(fg_batch* B, cudaStream_t st) {
  fg_engine* e = B->e;
  enqueue_all(B, st);  // warm-up; leaves a developed emulsion for the scan trials
  FG_CUDA(cudaStreamSynchronize(st));
  check_error_word(e);
  stage_bvh(B, st);  // the run ended with the scan's tree in the shared tree buffers
  float best = 1e30f;
  unsigned bb = B->tr_blocks, bt_ = B->tr_threads;
  for (unsigned threads : {128u, 256u}) {
    for (unsigned per_sm : {2u, 4u, 8u, 16u}) {
      const unsigned blocks = static_cast<unsigned>(e->sm_count) * per_sm * 256u / threads;
      B->tr_blocks = blocks;
      B->tr_threads = threads;
      FG_CUDA(cudaEventRecord(B->ev[2], st));
      stage_transport(B, st);
      FG_CUDA(cudaEventRecord(B->ev[3], st));
      FG_CUDA(cudaStreamSynchronize(st));
      const float ms = ev_ms(B->ev[2], B->ev[3]);
      if (ms < best) {
        best = ms;
        bb = blocks;
        bt_ = threads;
      }
    }
  }
  B->tr_blocks = bb;
  B->tr_threads = bt_;
  // Recreate the transport result of the chosen shape (counts are identical for every shape).
  stage_transport(B, st);
  stage_develop(B, st);
  best = 1e30f;
  uint32_t bp_best = B->bin_px;
  for (uint32_t bp : {4u, 8u}) {
    layout_bins(B, bp);
    upload_descriptors(B, st);
    FG_CUDA(cudaEventRecord(B->ev[4], st));
    stage_scan(B, st);
    FG_CUDA(cudaEventRecord(B->ev[5], st));
    FG_CUDA(cudaStreamSynchronize(st));
    const float ms = ev_ms(B->ev[4], B->ev[5]);
    if (ms < best) {
      best = ms;
      bp_best = bp;
    }
  }
  layout_bins(B, bp_best);
  upload_descriptors(B, st);
  FG_CUDA(cudaStreamSynchronize(st));
  check_error_word(e);
}

static void plan(fg_batch* B, const fg_batch_options* opt) {
  fg_engine* e = B->e;
  cudaStream_t st = e->stream;
  (void)cudaGetLastError();  // start from a clean runtime error state (library queries check it)
  const uint32_t n = B->ntiles;
  B->syn.resize(n);
  B->td.resize(n);
  B->sc.resize(n);
  B->bt.resize(n);
  B->exp_off.resize(n);
  B->out_off.resize(n);
  unsigned long long cb = 0, sb = 0, cap = 0, pb = 0, eo = 0, oo = 0;
  unsigned colc[4] = {0, 0, 0, 0};
  for (uint32_t i = 0; i < n; ++i) {
    derive_tile(B->params[i], B->syn[i], B->td[i], B->sc[i], B->bt[i]);
    SynthTile& s = B->syn[i];
    s.cell_base = cb;
    s.slot_base = sb;
    s.cbase = cap;
    for (int c = 0; c < 4; ++c) {
      s.col_base[c] = colc[c];
      const uint32_t cxn = (s.nbx + 1 - (c & 1)) / 2, cyn = (s.nby + 1 - (c >> 1)) / 2;
      colc[c] += cxn * cyn;
    }
    cb += static_cast<unsigned long long>(s.gw) * s.gh * s.gd;
    sb += 1ull << (2 * s.slot_bits);  // bricks
    B->maxcells = std::max<unsigned long long>(B->maxcells, static_cast<unsigned long long>(s.gw) * s.gh * s.gd);
    B->maxslots = std::max<unsigned long long>(B->maxslots, 1ull << (2 * s.slot_bits));
    cap += s.ccap;
    B->td[i].photon_base = pb;
    pb += B->td[i].P;
    {
      const double side = std::max(B->params[i].film_w, B->params[i].film_h) / PHOTON_CELL_UM;
      uint32_t bits = 0;
      while ((1u << bits) < static_cast<uint32_t>(std::ceil(side))) ++bits;
      B->td[i].pcell_bits = bits;
      B->td[i].pcell_base = static_cast<uint32_t>(B->npcells);
      B->npcells += 1ull << (2 * bits);
    }
    B->exp_off[i] = eo;
    eo += static_cast<unsigned long long>(B->params[i].width_px) * B->params[i].height_px;
    B->out_off[i] = oo;
    oo += static_cast<unsigned long long>(B->params[i].width_px) * B->params[i].height_px;
    B->gdmax = std::max<int>(B->gdmax, static_cast<int>(s.gd));
    B->rays += static_cast<unsigned long long>(B->sc[i].w) * B->sc[i].h * B->sc[i].spp;
  }
  for (int c = 0; c < 4; ++c) B->cols[c] = colc[c];
  FG_REQUIRE(cap < 0x7fffffffull, "batch too large: more than 2^31 crystal slots");
  FG_REQUIRE(bridson_smem(B->gdmax) <= 220 * 1024, "emulsion too deep for the synthesis column");
  B->ncells = cb;
  B->nslots = sb;
  B->ncap = cap;
  B->photons = pb;
  B->exp_total = eo;
  B->out_total = oo;
  B->tr_threads = opt && opt->transport_threads ? opt->transport_threads : 256;
  B->tr_blocks = opt && opt->transport_blocks ? opt->transport_blocks : static_cast<unsigned>(e->sm_count) * 8;
  const uint32_t bin0 = opt && opt->scan_bin_px ? opt->scan_bin_px : 8;
  B->use_graph = !opt || opt->use_graph;
  B->wait_limit = opt ? opt->synth_wait_limit : 0;
  B->wait_probe = opt && opt->wait_probe;
  if (B->wait_probe) {
    B->probe.alloc(1, st);
    FG_CUDA(cudaMemsetAsync(B->probe.p, 0, sizeof(uint32_t), st));
  }
  // Buffers (bins sized for the smallest bin edge the tuner tries).
  layout_bins(B, 4);
  const unsigned long long nbins_max = B->nbins;
  B->d_syn.alloc(n, st);
  B->d_td.alloc(n, st);
  B->d_sc.alloc(n, st);
  B->d_bt.alloc(n, st);
  B->cells.alloc(std::max<unsigned long long>(cb, 1), st);
  B->npts.alloc(n, st);
  B->coldone.alloc(std::max(B->cols[0] + B->cols[1] + B->cols[2] + B->cols[3], 1u), st);
  B->ncrys.alloc(n, st);
  B->flags.alloc(sb + 1, st);
  B->slot_scan.alloc(sb + 1, st);
  FG_CUDA(cudaMemsetAsync(B->slot_scan.p, 0, (sb + 1) * sizeof(uint32_t), st));  // n = 0 until the first run
  B->A.alloc(std::max<unsigned long long>(cap, 1), st);
  B->Q.alloc(std::max<unsigned long long>(cap, 1), st);
  B->D.alloc(std::max<unsigned long long>(cap, 1), st);
  B->EA.alloc(std::max<unsigned long long>(cap, 1), st);
  B->EQ.alloc(std::max<unsigned long long>(cap, 1), st);
  B->ED.alloc(std::max<unsigned long long>(cap, 1), st);
  B->keys.alloc(std::max<unsigned long long>(cap, 1), st);
  B->parent.alloc(std::max<unsigned long long>(cap, 1), st);
  B->counts.alloc(std::max<unsigned long long>(cap, 1), st);
  B->size.alloc(std::max<unsigned long long>(cap, 1), st);
  B->developed.alloc(std::max<unsigned long long>(cap, 1), st);
  B->exp64.alloc(std::max<unsigned long long>(cap, 1), st);
  {
    // Tree tiles: elements in the crystal-slot space (ebase = cbase), about 0.67 nodes per crystal.
    std::vector<RTile> rt(n), rs(n);
    for (uint32_t i = 0; i < n; ++i) {
      RTile& t = rt[i];
      t = RTile{};
      t.a = B->A.p + B->syn[i].cbase;
      t.d = B->D.p + B->syn[i].cbase;
      t.ecap = B->syn[i].ccap;
      t.pad = B->bt[i].pad;
      // The synthesis's radius clamp (emulsion.rs:162-170) for cubes; the other shapes lie in their boxes.
      t.reach = rt_reach(B->params[i].morphology == FG_CUBIC ? 0.48 * B->params[i].r_min : 0.0);
    }
    rtree_alloc(B->rt, rt, true, st, RT_NODE_FRAC);
    for (uint32_t i = 0; i < n; ++i) {
      FG_REQUIRE(rt[i].ebase == B->syn[i].cbase, "tree layout differs from the crystal slots");
      B->bt[i].nbase = rt[i].nbase;
      B->bt[i].ncap = rt[i].ncap;
      B->bt[i].rbase = rt[i].rbase;
      B->bt[i].rcap = rt[i].rcap;
      B->td[i].nnodes = rt[i].ncap;
      B->td[i].nrec = rt[i].rcap;
      B->td[i].reach = rt[i].reach;
      rs[i] = rt[i];
      rs[i].exp64 = B->exp64.p + B->syn[i].cbase;
    }
    B->rt_scan.alloc(n, st);
    FG_CUDA(cudaMemcpyAsync(B->rt_scan.p, rs.data(), n * sizeof(RTile), cudaMemcpyHostToDevice, st));
  }
  B->prep.alloc(std::max<unsigned long long>(cap, 1), st);
  B->devflag.alloc(cap + 1, st);
  B->devscan.alloc(cap + 1, st);
  B->devlist.alloc(std::max<unsigned long long>(cap, 1), st);
  B->bin_cnt.alloc(nbins_max + 1, st);
  B->bin_off.alloc(nbins_max + 1, st);
  B->bin_cur.alloc(nbins_max + 1, st);
  B->item_cap = std::max<unsigned long long>(cap * 8, 1);
  B->bin_items.alloc(B->item_cap, st);
  B->exposure.alloc(std::max<unsigned long long>(eo, 1), st);
  B->d_neg.alloc(std::max<unsigned long long>(oo, 1), st);
  B->counter.alloc(1, st);
  FG_REQUIRE(pb < 0xffffffffull && B->npcells < 0xffffffffull, "batch too large: photon count");
  B->pcnt.alloc(B->npcells + 1, st);
  B->poff.alloc(B->npcells + 1, st);
  B->pcur.alloc(B->npcells + 1, st);
  B->porder.alloc(std::max<unsigned long long>(pb, 1), st);
  B->dstats.alloc(4, st);
  FG_CUDA(cudaMemsetAsync(B->exposure.p, 0, B->exposure.n * sizeof(float), st));
  size_t b1 = 0, b2 = 0;
  FG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, b1, B->flags.p, B->slot_scan.p, static_cast<int64_t>(sb + 1), st));
  FG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, b2, B->bin_cnt.p, B->bin_off.p, static_cast<int64_t>(nbins_max + 1), st));
  size_t b3 = 0;
  FG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, b3, B->pcnt.p, B->poff.p, static_cast<int64_t>(B->npcells + 1), st));
  size_t b4 = 0;
  FG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, b4, B->devflag.p, B->devscan.p, static_cast<int64_t>(cap + 1), st));
  B->cub_bytes = std::max(std::max(b1, b2), std::max(b3, b4));
  B->cub_tmp.alloc(std::max<size_t>(B->cub_bytes, 1), st);
  for (auto& x : B->ev) FG_CUDA(cudaEventCreate(&x));
  layout_bins(B, bin0);
  upload_descriptors(B, st);
  FG_CUDA(cudaStreamSynchronize(st));
}

static void capture(fg_batch* B) {
  cudaStream_t st = B->e->stream;
  FG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    enqueue_all(B, st, true);
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(st, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  FG_CUDA(cudaStreamEndCapture(st, &B->graph));
  FG_CUDA(cudaGraphInstantiate(&B->exec, B->graph, 0));
}

unsigned long long tile_footprint(const fg_tile_params& p, unsigned long long* slots) {
  SynthTile s;
  TileDesc t;
  ScanTile c;
  BTile b;
  derive_tile(p, s, t, c, b);
  if (slots) *slots = s.ccap;
  const double side = std::max(p.film_w, p.film_h) / PHOTON_CELL_UM;
  uint32_t bits = 0;
  while ((1u << bits) < static_cast<uint32_t>(std::ceil(side))) ++bits;
  const unsigned long long px = static_cast<unsigned long long>(p.width_px) * p.height_px;
  // Per crystal slot: records 48 (and 48 in the tree's element order), key 8, links and flags 36, expansion 8, scan prep 160, bin
  // entries 32, tree elements 88 (order, node of, two copies of three 8-byte keys, flags, prefix
  // sums, ranks, final order, leaf of) and 0.8 nodes of 224 B (plus slack); cells 4 B; bricks
  // 8 B; photon order; images.
  return static_cast<unsigned long long>(s.ccap) * 628ull + static_cast<unsigned long long>(s.gw) * s.gh * s.gd * 4ull +
         (8ull << (2 * s.slot_bits)) + static_cast<unsigned long long>(t.P) * 4ull +
         (1ull << (2 * bits)) * 12ull + px * 8ull + 4096ull;
}

}  // namespace fg

extern "C" {

// VirtualEmulsionLayer::synthesize (emulsion.rs:155-220) on the device: the tile synthesis of this
// file over the whole emulsion as one tile, then the LBVH.  Crystal ids are the Morton slot order
// of the synthesis (the reference numbers crystals in its sampler's output order, which the random
// streams do not pin either).
fg_status fg_emulsion_synthesize(fg_engine* e, const fg_emulsion_cfg* cfg, uint64_t seed, fg_emulsion** out) {
  if (!out) return FG_ERR_INVALID_ARG;
  *out = nullptr;
  return guard(e, [&] {
    FG_REQUIRE(cfg, "null config");
    cudaStream_t st = e->stream;
    begin_call(e);
    (void)cudaGetLastError();
    fg_tile_params p{};
    p.film_w = cfg->width;
    p.film_h = cfg->height;
    p.film_d = cfg->depth;
    p.width_px = p.height_px = 1;
    p.seed = seed;
    p.r_min = cfg->r_min;
    p.mean_crystal_radius = cfg->mean_crystal_radius;
    p.size_variance = cfg->size_variance;
    p.morphology = cfg->morphology;
    p.tabular_aspect_ratio = cfg->tabular_aspect_ratio;
    p.base_sensitivity = cfg->base_sensitivity;
    SynthTile s;
    TileDesc td;
    ScanTile sc;
    BTile bt;
    derive_tile(p, s, td, sc, bt);
    const unsigned long long ncells = static_cast<unsigned long long>(s.gw) * s.gh * s.gd;
    FG_REQUIRE(s.ccap < 0x7ffffff0u, "emulsion too large");
    unsigned cols[4];
    for (int c = 0; c < 4; ++c) {
      s.col_base[c] = 0;
      cols[c] = ((s.nbx + 1 - (c & 1)) / 2) * ((s.nby + 1 - (c >> 1)) / 2);
    }
    const int gdmax = static_cast<int>(s.gd);
    FG_REQUIRE(bridson_smem(gdmax) <= 220 * 1024, "emulsion too deep for the synthesis column");
    FG_CUDA(cudaEventRecord(e->timer.ev[0], st));
    DBuf<SynthTile> d_syn(1, st);
    FG_CUDA(cudaMemcpyAsync(d_syn.p, &s, sizeof(SynthTile), cudaMemcpyHostToDevice, st));
    const unsigned long long nbr = 1ull << (2 * s.slot_bits);  // bricks
    DBuf<uint32_t> cells(ncells, st), npts(1, st), flags(nbr + 1ull, st), scan(nbr + 1ull, st);
    DBuf<float4> A(s.ccap, st), Q(s.ccap, st), D(s.ccap, st);
    DBuf<uint64_t> keys(s.ccap, st);
    FG_CUDA(cudaMemsetAsync(cells.p, 0, ncells * sizeof(uint32_t), st));
    FG_CUDA(cudaMemsetAsync(npts.p, 0, sizeof(uint32_t), st));
    DBuf<uint32_t> coldone(std::max(cols[0] + cols[1] + cols[2] + cols[3], 1u), st);
    launch_bridson(d_syn.p, 1, cols, gdmax, cells.p, npts.p, coldone.p, e->d_err, st);
    FG_CUDA(cudaMemsetAsync(flags.p + nbr, 0, sizeof(uint32_t), st));
    launch_synth_post(d_syn.p, 1, ncells, nbr, cells.p, npts.p, flags.p, st);
    exclusive_scan_u32(flags.p, scan.p, nbr + 1ull, st);
    launch_emit(d_syn.p, 1, nbr, cells.p, scan.p, A.p, Q.p, D.p, keys.p, e->d_err, st);
    uint32_t n = 0;
    FG_CUDA(cudaMemcpyAsync(&n, scan.p + nbr, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    check_error_word(e);
    n = std::min(n, s.ccap);
    std::unique_ptr<fg_emulsion> em(new fg_emulsion());
    em->cfg = *cfg;
    em->n = n;
    em->stream = st;
    em->has64 = false;
    em->extent = std::max(std::max(cfg->width, cfg->height), cfg->depth);
    em->max_half_dim = 0.48 * cfg->r_min;  // the radius clamp of the synthesis (emulsion.rs:162-170)
    em->any_cubic = cfg->morphology == FG_CUBIC;
    em->a = std::move(A);
    em->q = std::move(Q);
    em->d = std::move(D);
    alloc_state(em.get(), st);
    DBuf<uint32_t> none;
    build_emulsion_tree(e, em.get(), false, em->rt, none);
    FG_CUDA(cudaEventRecord(e->timer.ev[1], st));
    FG_CUDA(cudaStreamSynchronize(st));
    e->timings.synth_ms = elapsed(e->timer.ev[0], e->timer.ev[1]);
    e->timings.total_ms = e->timings.synth_ms;
    e->timings.crystals = n;
    end_call(e);
    *out = em.release();
  });
}

fg_status fg_tile_params_preset(const char* preset, double pixel_size_um, uint32_t tw, uint32_t th,
                                double exposure, double push, uint64_t tile_seed, fg_tile_params* out) {
  if (!preset || !out || !(pixel_size_um > 0) || tw == 0 || th == 0) return FG_ERR_INVALID_ARG;
  std::string s(preset);
  for (auto& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
  const bool is1600 = s.find("1600") != std::string::npos || s == "caffenol";
  const double eff_push = is1600 ? std::max(push, 2.0) : std::max(push, 0.0);  // image_pipeline.rs:369-375
  // Emulsion stock of the tile worker (image_pipeline.rs:925-938): tri-x at push >= 1.5 uses 1600.
  std::string stock;
  if (s == "t-max" || s == "tmax") stock = "t-max";
  else if (s == "hp5" || s == "hp5-plus") stock = "hp5";
  else if (is1600) stock = "tri-x-1600";
  else stock = eff_push >= 1.5 ? "tri-x-1600" : "tri-x";
  fg_emulsion_cfg ec;
  const fg_status st = fg_emulsion_preset(stock.c_str(), tw * pixel_size_um, th * pixel_size_um, &ec);
  if (st != FG_OK) return st;
  *out = fg_tile_params{};
  out->film_w = ec.width;
  out->film_h = ec.height;
  out->film_d = ec.depth;
  out->width_px = tw;
  out->height_px = th;
  out->samples_per_pixel = 4;       // render_tile_cpu_density, image_pipeline.rs:996-1002
  out->threshold_photons = 4;       // image_pipeline.rs:964
  out->silver_opacity = 0.25;
  out->seed = tile_seed;
  out->r_min = ec.r_min;
  out->mean_crystal_radius = ec.mean_crystal_radius;
  out->size_variance = ec.size_variance;
  out->morphology = ec.morphology;
  out->tabular_aspect_ratio = ec.tabular_aspect_ratio;
  out->base_sensitivity = ec.base_sensitivity;
  out->exposure = exposure;
  if (s == "t-max" || s == "tmax") {
    out->filament_expansion = 1.10 + 0.04 * eff_push;
    out->clumping_proximity_factor = 1.10 + 0.03 * eff_push;
  } else if (s == "hp5" || s == "hp5-plus") {
    out->filament_expansion = 1.15 + 0.05 * eff_push;
    out->clumping_proximity_factor = 1.18 + 0.04 * eff_push;
  } else {
    out->filament_expansion = 1.20 + 0.06 * eff_push;
    out->clumping_proximity_factor = 1.25 + 0.05 * eff_push;
  }
  out->optics = ec.optics;
  out->photons_per_sq_um = 6.0;     // image_pipeline.rs:943
  out->illumination_angle_rad = 0.12;
  out->crystal_absorption_coeff = 1.3;
  out->max_bounces = 48;
  return FG_OK;
}

fg_status fg_batch_create(fg_engine* e, const fg_tile_params* tiles, uint32_t ntiles,
                          const fg_batch_options* opt, fg_batch** out) {
  if (!out) return FG_ERR_INVALID_ARG;
  *out = nullptr;
  return guard(e, [&] {
    FG_REQUIRE(tiles && ntiles > 0, "no tiles");
    std::unique_ptr<fg_batch> B(new fg_batch());
    B->e = e;
    B->ntiles = ntiles;
    B->params.assign(tiles, tiles + ntiles);
    plan(B.get(), opt);
    if (opt && opt->autotune) {
      B->tune_pending = true;  // tuned on the first run's exposure, then captured
    } else if (B->use_graph) {
      capture(B.get());
    }
    *out = B.release();
  });
}

fg_status fg_batch_destroy(fg_batch* b) {
  if (!b) return FG_ERR_INVALID_ARG;
  fg_engine* e = b->e;
  return guard(e, [&] {
    FG_CUDA(cudaStreamSynchronize(e->stream));
    delete b;
    FG_CUDA(cudaStreamSynchronize(e->stream));
  });
}

fg_status fg_batch_set_exposure(fg_batch* b, const float* const* tiles) {
  if (!b) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    FG_REQUIRE(tiles, "null tile list");
    for (uint32_t i = 0; i < b->ntiles; ++i) {
      FG_REQUIRE(tiles[i], "null exposure tile");
      const size_t n = static_cast<size_t>(b->params[i].width_px) * b->params[i].height_px;
      FG_CUDA(cudaMemcpyAsync(b->exposure.p + b->exp_off[i], tiles[i], n * sizeof(float), cudaMemcpyHostToDevice,
                              b->e->stream));
    }
  });
}

fg_status fg_batch_exposure_device(fg_batch* b, uint32_t tile, float** ptr) {
  if (!b || !ptr || tile >= b->ntiles) return FG_ERR_INVALID_ARG;
  *ptr = b->exposure.p + b->exp_off[tile];
  return FG_OK;
}

fg_status fg_batch_density_device(fg_batch* b, uint32_t tile, const float** ptr) {
  if (!b || !ptr || tile >= b->ntiles) return FG_ERR_INVALID_ARG;
  *ptr = b->d_neg.p + b->out_off[tile];
  return FG_OK;
}

// First run of an autotuned batch: time the candidates on the exposure now set, then capture.
static void finish_setup(fg_batch* B) {
  if (!B->tune_pending) return;
  autotune(B, B->e->stream);
  if (B->use_graph) capture(B);
  B->tune_pending = false;
}

fg_status fg_batch_run(fg_batch* b) {
  if (!b) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    cudaStream_t st = b->e->stream;
    finish_setup(b);
    if (b->exec) {
      FG_CUDA(cudaGraphLaunch(b->exec, st));
    } else {
      enqueue_all(b, st);
    }
  });
}

fg_status fg_batch_wait(fg_batch* b, fg_batch_stats* stats) {
  if (!b) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    cudaStream_t st = b->e->stream;
    FG_CUDA(cudaStreamSynchronize(st));
    check_error_word(b->e);
    fg_batch_stats s{};
    s.synth_ms = ev_ms(b->ev[0], b->ev[1]);
    s.bridson_ms = ev_ms(b->ev[8], b->ev[7]);
    s.bvh_ms = ev_ms(b->ev[1], b->ev[2]);
    s.transport_ms = ev_ms(b->ev[2], b->ev[3]);
    s.develop_ms = ev_ms(b->ev[3], b->ev[4]);
    s.scan_ms = ev_ms(b->ev[4], b->ev[5]);
    s.total_ms = ev_ms(b->ev[0], b->ev[5]);
    std::vector<uint32_t> nc(b->ntiles);
    FG_CUDA(cudaMemcpy(nc.data(), b->ncrys.p, b->ntiles * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (uint32_t v : nc) s.crystals += v;
    s.photons = b->photons;
    unsigned long long ds[4];
    FG_CUDA(cudaMemcpy(ds, b->dstats.p, sizeof(ds), cudaMemcpyDeviceToHost));
    s.hits = ds[0];
    s.scan_fallbacks = ds[1];
    s.scan_hits = ds[2];
    s.clumps = ds[3];
    uint32_t ndev = 0;  // the exclusive scan of the developed flags ends with their total
    FG_CUDA(cudaMemcpy(&ndev, b->devscan.p + b->ncap, sizeof(ndev), cudaMemcpyDeviceToHost));
    s.developed = ndev;
    s.cells = b->ncells;
    s.rays = b->rays;
    s.pixels = b->out_total;
    s.transport_threads = b->tr_threads;
    s.transport_blocks = b->tr_blocks;
    s.scan_bin_px = b->bin_px;
    s.graph = b->exec ? 1u : 0u;
    // Own kernels per run: Bridson (all colour classes in one launch; it also counts the points), thin +
    // brick counts, emit, set_n, photon order x2, transport, maxdim + threshold + developed list + link +
    // roots + finalize, scan-tree inputs, scan prep, two bin passes, scan, density, the crystal records in
    // the transport tree's order, and the two tree builds (each level's launches included, also those that
    // find no work; CUB scans not counted).
    s.kernel_launches = 1 + 2 + 1 + 1 + 2 + 1 + 6 + 1 + 1 + 2 + 1 + 1 + 1 + 2 * rtree_kernel_launches(b->rt);
    b->stats = s;
    if (stats) *stats = s;
  });
}

fg_status fg_batch_get_density(fg_batch* b, float* const* outs) {
  if (!b) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    FG_REQUIRE(outs, "null output list");
    for (uint32_t i = 0; i < b->ntiles; ++i) {
      FG_REQUIRE(outs[i], "null output tile");
      const size_t n = static_cast<size_t>(b->params[i].width_px) * b->params[i].height_px;
      FG_CUDA(cudaMemcpyAsync(outs[i], b->d_neg.p + b->out_off[i], n * sizeof(float), cudaMemcpyDeviceToHost,
                              b->e->stream));
    }
    FG_CUDA(cudaStreamSynchronize(b->e->stream));
  });
}

fg_status fg_batch_tile_crystals(fg_batch* b, uint32_t tile, fg_crystals_out* out, uint32_t* counts,
                                 uint8_t* developed, double* expansion, size_t cap, size_t* n) {
  if (!b || tile >= b->ntiles || !n) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    cudaStream_t st = b->e->stream;
    uint32_t nc = 0;
    FG_CUDA(cudaMemcpyAsync(&nc, b->ncrys.p + tile, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    *n = nc;
    const size_t k = std::min<size_t>(nc, cap);
    if (!k) return;
    const unsigned long long cb = b->syn[tile].cbase;
    std::vector<float4> A(k), Q(k), D(k);
    FG_CUDA(cudaMemcpyAsync(A.data(), b->A.p + cb, k * sizeof(float4), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(Q.data(), b->Q.p + cb, k * sizeof(float4), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaMemcpyAsync(D.data(), b->D.p + cb, k * sizeof(float4), cudaMemcpyDeviceToHost, st));
    if (counts) FG_CUDA(cudaMemcpyAsync(counts, b->counts.p + cb, k * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (developed) FG_CUDA(cudaMemcpyAsync(developed, b->developed.p + cb, k, cudaMemcpyDeviceToHost, st));
    if (expansion) FG_CUDA(cudaMemcpyAsync(expansion, b->exp64.p + cb, k * sizeof(double), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    for (size_t i = 0; i < k; ++i) {
      if (out && out->pos) { out->pos[3 * i] = A[i].x; out->pos[3 * i + 1] = A[i].y; out->pos[3 * i + 2] = A[i].z; }
      if (out && out->dims) { out->dims[3 * i] = D[i].x; out->dims[3 * i + 1] = D[i].y; out->dims[3 * i + 2] = D[i].z; }
      if (out && out->quat) { out->quat[4 * i] = Q[i].x; out->quat[4 * i + 1] = Q[i].y; out->quat[4 * i + 2] = Q[i].z; out->quat[4 * i + 3] = Q[i].w; }
      if (out && out->sensitivity) out->sensitivity[i] = A[i].w;
      if (out && out->morphology) { int32_t m; std::memcpy(&m, &D[i].w, 4); out->morphology[i] = m; }
    }
  });
}

fg_status fg_batch_time(fg_batch* b, uint32_t steps, double* ms) {
  if (!b || !ms || steps == 0) return FG_ERR_INVALID_ARG;
  return guard(b->e, [&] {
    cudaStream_t st = b->e->stream;
    finish_setup(b);
    FG_CUDA(cudaStreamSynchronize(st));
    FG_CUDA(cudaEventRecord(b->ev[6], st));
    for (uint32_t i = 0; i < steps; ++i) {
      if (b->exec) {
        FG_CUDA(cudaGraphLaunch(b->exec, st));
      } else {
        enqueue_all(b, st);
      }
    }
    FG_CUDA(cudaEventRecord(b->ev[5], st));
    FG_CUDA(cudaStreamSynchronize(st));
    check_error_word(b->e);
    *ms = ev_ms(b->ev[6], b->ev[5]);
  });
}

fg_status fg_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return FG_ERR_INVALID_ARG;
  *ptr = nullptr;
  if (cudaMallocHost(ptr, bytes ? bytes : 1) != cudaSuccess) return FG_ERR_OOM;
  return FG_OK;
}

fg_status fg_host_free(void* ptr) {
  if (ptr && cudaFreeHost(ptr) != cudaSuccess) return FG_ERR_INVALID_ARG;
  return FG_OK;
}

fg_status fg_render_batch(fg_engine* e, const fg_tile_params* tiles, uint32_t ntiles, const float* const* exposure,
                          float* const* d_neg) {
  fg_batch* b = nullptr;
  fg_batch_options opt{};
  opt.use_graph = 0;
  fg_status s = fg_batch_create(e, tiles, ntiles, &opt, &b);
  if (s != FG_OK) return s;
  s = fg_batch_set_exposure(b, exposure);
  if (s == FG_OK) s = fg_batch_run(b);
  if (s == FG_OK) s = fg_batch_wait(b, nullptr);
  if (s == FG_OK) s = fg_batch_get_density(b, d_neg);
  const fg_status d = fg_batch_destroy(b);
  return s != FG_OK ? s : d;
}

fg_status fg_render_tile(fg_engine* e, const float* tile, const fg_tile_params* p, float* d_neg) {
  if (!p || !tile || !d_neg) return FG_ERR_INVALID_ARG;
  return fg_render_batch(e, p, 1, &tile, &d_neg);
}

}  // extern "C"
