// Host-side internals shared by the translation units of libfgrain_cuda.so.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/fgrain_cuda.h"
#include "fg_device.cuh"
#include "fg_rtree.cuh"

namespace fg {

// A failed CUDA call or a rejected argument, carried to the C boundary as (status, message).
struct Error {
  fg_status st;
  std::string msg;
};

#define FG_CUDA(call)                                                                     \
  do {                                                                                    \
    cudaError_t e__ = (call);                                                             \
    if (e__ != cudaSuccess) throw ::fg::Error{::fg::status_of(e__), std::string(#call) + \
                                              ": " + cudaGetErrorString(e__)};            \
  } while (0)

#define FG_REQUIRE(cond, msg)                                                   \
  do {                                                                          \
    if (!(cond)) throw ::fg::Error{FG_ERR_INVALID_ARG, std::string(msg)};       \
  } while (0)

inline fg_status status_of(cudaError_t e) {
  switch (e) {
    case cudaErrorMemoryAllocation: return FG_ERR_OOM;
    case cudaErrorInvalidDevice:
    case cudaErrorNoDevice:
    case cudaErrorInsufficientDriver: return FG_ERR_ADAPTER_NOT_FOUND;
    case cudaErrorInvalidValue: return FG_ERR_INVALID_ARG;
    default: return FG_ERR_PIPELINE;
  }
}

// Device bytes held through DBuf and the optional cap on them (fg_set_device_budget).
inline std::atomic<unsigned long long> g_dev_bytes{0};
inline std::atomic<unsigned long long> g_dev_budget{0};

// Device buffer owned by RAII; stream-ordered allocation on the engine stream.  view() makes it a
// non-owning window onto memory that someone else holds (nothing is freed then).
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;
  bool own = true;
  DBuf() = default;
  DBuf(size_t count, cudaStream_t st) { alloc(count, st); }
  void alloc(size_t count, cudaStream_t st) {
    release();
    s = st;
    own = true;
    if (!count) return;
    const unsigned long long bytes = count * sizeof(T), cap = g_dev_budget.load();
    if (cap && g_dev_bytes.fetch_add(bytes) + bytes > cap) {
      g_dev_bytes.fetch_sub(bytes);
      throw Error{FG_ERR_OOM, "device budget of " + std::to_string(cap) + " bytes exceeded (fg_set_device_budget)"};
    }
    if (!cap) g_dev_bytes.fetch_add(bytes);
    const cudaError_t r = cudaMallocAsync(reinterpret_cast<void**>(&p), bytes, st);
    if (r != cudaSuccess) {
      g_dev_bytes.fetch_sub(bytes);
      p = nullptr;
      throw Error{status_of(r), std::string("cudaMallocAsync: ") + cudaGetErrorString(r)};
    }
    n = count;
  }
  void view(T* ptr, size_t count) {
    release();
    p = ptr;
    n = count;
    own = false;
  }
  void release() {
    if (p && own) {
      cudaFreeAsync(p, s);
      g_dev_bytes.fetch_sub(n * sizeof(T));
    }
    p = nullptr;
    n = 0;
    own = true;
  }
  ~DBuf() { release(); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), s(o.s), own(o.own) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; s = o.s; own = o.own; o.p = nullptr; o.n = 0; }
    return *this;
  }
};

// Stage timer: events recorded on the engine stream around each stage.
struct StageTimer {
  cudaEvent_t ev[2 * 8];
  int used = 0;
  bool made = false;
  void init() {
    if (made) return;
    for (auto& e : ev) FG_CUDA(cudaEventCreate(&e));
    made = true;
  }
  void destroy() {
    if (!made) return;
    for (auto& e : ev) cudaEventDestroy(e);
    made = false;
  }
};

// fg_rtree.cu: device buffers of reference-tree builds over the tiles of a batch (or one
// emulsion).  Element positions and nodes are laid out tile after tile (RTile::ebase, nbase).
struct RTreeBufs {
  int ntiles = 0;
  int levels = 0;                 // global split levels before the per-warp finish
  unsigned long long E = 0, N = 0, nblk = 0;
  uint32_t count = 0;             // elements of a one-tile tree built on the host's request
  DBuf<RTile> tiles;
  DBuf<uint32_t> idx0, idx1, nof0, nof1, flag, bb, blk, P, Q;
  DBuf<unsigned long long> key0, key1;  // three ordered centroid keys per element (SoA), travelling with the order
  DBuf<uint32_t> ridx;            // final element order (slots): a leaf's crystals in reference order
  DBuf<unsigned long long> acc;   // per node: ordered centroid minima, maxima (3 each)
  DBuf<double> box64;             // per node: lo xyz, hi xyz (FP64, exact)
  DBuf<uint32_t> parent;          // per node: parent id (0xffffffff for a root)
  DBuf<uint32_t> nstart, ncount, ntile, ndepth;
  DBuf<int> nsplit;               // split axis, -1 for a leaf
  DBuf<double> nmid;
  DBuf<int2> nchild;              // global ids of the children
  DBuf<uint32_t> wl0, wl1, bq, bqpar, cnt;  // global worklists (wl0 then the refit's arrival counts),
                                            // block queue (node, buffer parity), counts
  unsigned long long R = 0;       // walk records (all tiles)
  DBuf<Node4> rnode;              // four-wide walk records (tile-local refs)
  DBuf<uint2> rleaf;              // leaf: first element (tile-local position), count
  DBuf<uint32_t> leafof;          // optional: leaf id of each element slot
};
}  // namespace fg

struct fg_engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::recursive_mutex mu;
  std::string err;
  std::string name;
  uint32_t* d_err = nullptr;                    // device error word
  unsigned long long* d_stats = nullptr;        // device counters (hits, fallbacks, ...)
  fg_timings timings{};
  int sm_count = 0;
  fg::StageTimer timer;
};

struct fg_emulsion {
  fg_emulsion_cfg cfg{};
  uint32_t n = 0;
  cudaStream_t stream = nullptr;
  // Hot crystal records in Morton order.
  fg::DBuf<float4> a, q, d;
  // FP64 copies (uploaded sets only).
  fg::DBuf<double> pos64, dims64, quat64, sens64;
  fg::DBuf<uint32_t> sorted_to_id, id_to_sorted;
  // The reference tree over all crystals in id order (the transport walks, the development's
  // radius queries).
  fg::RTreeBufs rt;
  // Mutable per-crystal state (Morton order).
  fg::DBuf<uint32_t> counts;
  fg::DBuf<uint8_t> developed;
  fg::DBuf<float> exp32;
  fg::DBuf<double> exp64;
  fg::DBuf<int64_t> clump;  // by crystal id
  bool has64 = false;
  double extent = 0.0;             // largest coordinate magnitude (sets the box padding)
  double max_half_dim = 0.0;       // largest crystal half-dimension (sets the walks' reach)
  bool any_cubic = true;           // some crystal is a cube (only a cube reaches out of its box)
  std::vector<uint32_t> h_s2id;    // host copy of sorted_to_id (empty: identity)

  fg::CrystalsView view() const {
    fg::CrystalsView v;
    v.a = a.p; v.q = q.p; v.d = d.p;
    v.pos64 = has64 ? pos64.p : nullptr;
    v.dims64 = has64 ? dims64.p : nullptr;
    v.quat64 = has64 ? quat64.p : nullptr;
    v.sens64 = has64 ? sens64.p : nullptr;
    v.n = n;
    return v;
  }
};

namespace fg {

// fg_bvh.cu
// Sorts crystals by Morton code and fills the hot arrays; returns the sorted keys.
// pos_host / pos_dev: id-ordered FP64 positions on the host and on the device.
void morton_order(fg_emulsion* em, const double* pos_host, const double* pos_dev, cudaStream_t st,
                  DBuf<uint64_t>& keys, DBuf<uint32_t>& order);
void gather_sorted(fg_emulsion* em, const uint32_t* order, const double* pos, const double* dims,
                   const double* quat, const double* sens, const int32_t* morph, int32_t morph_all,
                   cudaStream_t st);

// Sets RTile::ebase / nbase / ncap from ecap, copies the tiles to the device and allocates.  The
// caller fills the source pointers and ecap of each tile, and RTile::n (and order) on the device
// before each build.
// Each tile gets min(ecap + 2, node_frac * ecap + 64) nodes (the reference tree has about 0.67
// nodes per element; running out fails the build with the list-overflow error bit).
// leafof (when wanted) gets max(elements, leafof_slots) words: it is indexed by element slot.
void rtree_alloc(RTreeBufs& B, std::vector<RTile>& tiles, bool want_leafof, cudaStream_t st, double node_frac = 1.0,
                 size_t leafof_slots = 0);
// Enqueues a build (capturable: no host synchronisation).  tiles_dev (optional) replaces the tile
// array of the allocation by one with the same layout (ebase, nbase, ecap, ncap) but other element
// sources, so that one set of buffers serves several trees in turn.
void rtree_build(RTreeBufs& B, uint32_t* err, cudaStream_t st, RTile* tiles_dev = nullptr);
unsigned rtree_kernel_launches(const RTreeBufs& B);
// One tile's build in memory the caller holds (nothing allocated): bytes needed for a tile of ecap
// elements, and the attach that carves every buffer (the tile descriptor too) from `base`
// (256-byte aligned).  The tile's source pointers are set by the caller; tile.n may be written on
// the device later (RTreeBufs::tiles.p).
size_t rtree_scratch_bytes(uint32_t ecap, bool want_leafof, uint32_t leafof_slots);
void rtree_attach(RTreeBufs& B, RTile tile, bool want_leafof, uint32_t leafof_slots, unsigned char* base,
                  size_t bytes, cudaStream_t st);
// The tree of an emulsion over all its crystals, or over its developed crystals with their
// expansion (the scan's tree, transmittance.rs:86-89), elements in crystal-id order.  list keeps
// the developed element list alive for the build.
void build_emulsion_tree(fg_engine* e, const fg_emulsion* em, bool developed_only, RTreeBufs& B,
                         DBuf<uint32_t>& list);

// fg_develop.cu
void develop(fg_engine* e, fg_emulsion* em, const fg_dev_cfg& cfg, fg_dev_report* rep);

// fg_scan.cu
struct ScanOut {
  float* out = nullptr;      // mode-mapped value per pixel
  uint8_t* image8 = nullptr; // 8-bit image
  float* d_neg = nullptr;    // -log10(clamp(T)) + 0.05
  uint16_t* ray_hits = nullptr;
};
// Host permutation helpers between crystal id order and Morton order.
template <class T>
std::vector<T> to_sorted(const fg_emulsion* em, const T* by_id) {
  std::vector<T> v(em->n);
  for (uint32_t s = 0; s < em->n; ++s) v[s] = by_id[em->h_s2id.empty() ? s : em->h_s2id[s]];
  return v;
}
template <class T>
void from_sorted(const fg_emulsion* em, const std::vector<T>& sorted, T* by_id) {
  for (uint32_t s = 0; s < em->n; ++s) by_id[em->h_s2id.empty() ? s : em->h_s2id[s]] = sorted[s];
}

// fg_image.cu: the separable 3-tap clamp-to-edge filter (two passes through tmp), in the
// reference's FP32 operation order, the second pass scaled by `scale`.
void launch_otf(const float* in, float* tmp, float* out, uint32_t w, uint32_t h, const float k[3], float scale,
                cudaStream_t st);

// Device bytes a batch needs for one tile (fg_batch.cu), a little above what plan() allocates;
// *slots (may be null) receives the tile's crystal slots.
unsigned long long tile_footprint(const fg_tile_params& p, unsigned long long* slots);

// Device state of a new emulsion (counts, development, clumps), zeroed (fg_engine.cu).
void alloc_state(fg_emulsion* em, cudaStream_t st);

// Per-call bookkeeping of the engine entry points (fg_engine.cu): zero the timings and device
// counters; read the counters back, synchronise and raise the device error word.
void begin_call(fg_engine* e);
void end_call(fg_engine* e);
float elapsed(cudaEvent_t a, cudaEvent_t b);

void scan(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
          const float* sigma_sorted, const ScanOut& out);
// g_sorted[s] += sum over the rays of each pixel p of wpx[p] / spp * T_ray * chord_s (device
// arrays; wpx has one weight per pixel, g_sorted one FP64 sum per crystal in Morton order).
void scan_adjoint(fg_engine* e, const fg_emulsion* em, const fg_scan_cfg& cfg, uint64_t seed,
                  const float* sigma_sorted, const float* wpx, double* g_sorted);

// fg_transport.cu
void expose(fg_engine* e, fg_emulsion* em, const float* tile_dev, uint32_t tw, uint32_t th,
            const fg_exposure_cfg& cfg, uint64_t seed, unsigned long long* photons_out);

// Exclusive prefix sum on the device (CUB).
void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t st);

// Raises an Error when a kernel reported one through the engine's error word.
void check_error_word(fg_engine* e);

// Runs f under the engine lock with the device current; converts failures to a status.
template <class F>
fg_status guard(fg_engine* e, F&& f) {
  if (!e) return FG_ERR_INVALID_ARG;
  std::lock_guard<std::recursive_mutex> lk(e->mu);
  try {
    FG_CUDA(cudaSetDevice(e->device));
    f();
    return FG_OK;
  } catch (const Error& x) {
    e->err = x.msg;
    return x.st;
  } catch (const std::bad_alloc&) {
    e->err = "host allocation failed";
    return FG_ERR_OOM;
  } catch (const std::exception& x) {
    e->err = x.what();
    return FG_ERR_PIPELINE;
  }
}

inline unsigned grid_for(size_t n, unsigned block) {
  return static_cast<unsigned>((n + block - 1) / block);
}

}  // namespace fg
