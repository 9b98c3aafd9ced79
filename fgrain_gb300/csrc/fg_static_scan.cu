// Transmittance scan that allocates no device memory: fg_scan_crystals_static.
//
// Who needs it: callers that own every byte of device memory they use and cannot let a library
// call cudaMalloc / cudaFree (or a stream-ordered or caching allocator) on their behalf.  Typical
// cases are a host application that runs under a fixed device-memory budget or its own pool
// allocator, a plugin loaded into such a host, and code that must not pay the implicit
// device-wide synchronisation of cudaMalloc / cudaFree.  Such a caller hands over the crystal set
// and the output image in device memory it already holds.
//
// The scan's own scratch (the reference tree over the developed crystals, bin lists, the kernel
// descriptor, the error word) lives in one file-scope __device__ array of
// FG_STATIC_SCAN_SCRATCH_BYTES (about 17 MB).  Every GPU on which this library is loaded holds that
// array until the process exits.  It bounds the work of one call: at most
// FG_STATIC_SCAN_MAX_CRYSTALS crystals of which FG_STATIC_SCAN_MAX_DEVELOPED developed,
// FG_STATIC_SCAN_MAX_BINS scan bins and FG_STATIC_SCAN_MAX_ITEMS (crystal, bin) entries; larger
// requests are rejected before any output is written.
//
// All calls on a device share the one array, and it keeps whatever the last call left in it:
// each call clears the parts that must start at zero (bin counts, cursors, error word) on the
// caller's stream.  Two calls whose GPU work overlapped (two host threads, or two streams) would
// race on the array and give wrong images.  The library prevents that within a process: a call
// holds a per-device lock from its first enqueue until its GPU work has finished (it synchronises
// the stream before it returns, also on failure), so concurrent callers wait for each other.
// Other processes load their own copy of the array.
//
// The tree, the bins, the binned scan kernel and the result are those of fg_scan_emulsion (same
// kernels, same descriptor), so both entry points give the same image for the same crystals.  The
// developed crystals enter the tree in whatever order the device lists them: the leaves' crystal
// sets and boxes, which are all the scan uses, do not depend on that order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "fg_internal.h"
#include "fg_scan.cuh"

namespace fg {

// Binning kernels and the scan launcher of fg_scan.cu.
__global__ void k_bin_count(ScanTile t, uint32_t* cnt);
__global__ void k_bin_fill(ScanTile t, const uint32_t* off, uint32_t* cursor, uint32_t* items);
void launch_scan(const ScanTile* tiles, int ntiles, unsigned long long nbins, unsigned threads, uint32_t* err,
                 unsigned long long* stats, cudaStream_t st);
uint32_t scan_bin_px(uint32_t spp);

namespace {

constexpr size_t round256(size_t v) { return (v + 255) / 256 * 256; }

// Scratch layout (byte offsets from the start of the array).
constexpr size_t kDescOff = 0;                                   // ScanTile descriptor
constexpr size_t kErrOff = 256;                                  // error word (+ 3 spare words)
constexpr size_t kBinBytes = round256((FG_STATIC_SCAN_MAX_BINS + 1ull) * sizeof(uint32_t));
constexpr size_t kCntOff = 512;                                  // per-bin counts, then total
constexpr size_t kOffOff = kCntOff + kBinBytes;                  // exclusive prefix sums
constexpr size_t kCurOff = kOffOff + kBinBytes;                  // fill cursors
constexpr size_t kItemsOff = kCurOff + kBinBytes;                // bin lists (crystal indices)
constexpr size_t kDevListOff = round256(kItemsOff + FG_STATIC_SCAN_MAX_ITEMS * sizeof(uint32_t));  // developed
constexpr size_t kDevCountOff = round256(kDevListOff + FG_STATIC_SCAN_MAX_DEVELOPED * sizeof(uint32_t));
constexpr size_t kTreeOff = kDevCountOff + 256;                  // the scan's reference tree
constexpr size_t kTreeBytes = rtree_attach_bytes(FG_STATIC_SCAN_MAX_DEVELOPED, true, FG_STATIC_SCAN_MAX_CRYSTALS);
constexpr size_t kScratchBytes = kTreeOff + kTreeBytes;
static_assert(sizeof(ScanTile) <= kErrOff - kDescOff, "scan descriptor does not fit its slot");
static_assert(kScratchBytes == FG_STATIC_SCAN_SCRATCH_BYTES, "header and scratch layout disagree");

}  // namespace

// The scratch itself.  On the host this name only identifies the symbol; its device address is
// looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_static_scan_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_call_mu[kMaxDevices];  // one per device: held for the whole of a call on that device

int current_device() {
  int dev = -1;
  FG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error{FG_ERR_ADAPTER_NOT_FOUND, "device ordinal out of range"};
  return dev;
}

// Device address of the scratch on device `dev` (the current device); the first call on a device
// looks it up.
unsigned char* scratch_for_device(int dev) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t r = cudaGetSymbolAddress(&p, g_static_scan_scratch);
    if (r != cudaSuccess || !p)
      throw Error{FG_ERR_DEVICE_REQUEST_FAILED,
                  std::string("cudaGetSymbolAddress(static scan scratch): ") + cudaGetErrorString(r)};
    g_scratch_addr[dev] = p;
  }
  return static_cast<unsigned char*>(g_scratch_addr[dev]);
}

// Exclusive prefix sum of n <= FG_STATIC_SCAN_MAX_BINS + 1 counts in one CTA of 1024 threads:
// each thread sums a contiguous run, the run totals are scanned across the CTA, then each thread
// writes its run's prefixes.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_exclusive_scan_small(const uint32_t* in, uint32_t* out,
                                                                       uint32_t n) {
  __shared__ uint32_t warp_tot[kScanThreads / 32];
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t per = (n + kScanThreads - 1) / kScanThreads;
  const uint32_t b = min(tid * per, n), e = min(b + per, n);
  uint32_t run = 0;
  for (uint32_t i = b; i < e; ++i) run += in[i];
  uint32_t incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= static_cast<uint32_t>(o)) incl += v;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= static_cast<uint32_t>(o)) w += v;
    }
    warp_tot[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint32_t acc = incl - run + (warp > 0 ? warp_tot[warp - 1] : 0u);
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t v = in[i];
    out[i] = acc;
    acc += v;
  }
}

// Lists the developed crystals (any order) and counts them; entries past `cap` are only counted.
__global__ void k_static_devlist(const uint8_t* developed, uint32_t n, uint32_t* list, uint32_t* count, uint32_t cap) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n || !developed[s]) return;
  const uint32_t k = atomicAdd(count, 1u);
  if (k < cap) list[k] = s;
}

void write_message(char* msg, size_t len, const std::string& s) {
  if (!msg || len == 0) return;
  const size_t k = std::min(len - 1, s.size());
  std::memcpy(msg, s.data(), k);
  msg[k] = '\0';
}

void static_scan(const fg_device_crystals* c, const fg_emulsion_cfg* film, const fg_scan_cfg* cfg,
                 uint64_t seed, float* out, uint8_t* image8, cudaStream_t st) {
  FG_REQUIRE(c && film && cfg, "null argument");
  FG_REQUIRE(out || image8, "no output: pass out and/or image8 (device pointers)");
  FG_REQUIRE(c->n <= FG_STATIC_SCAN_MAX_CRYSTALS,
             "too many crystals: the static scratch holds at most " + std::to_string(FG_STATIC_SCAN_MAX_CRYSTALS));
  if (c->n) FG_REQUIRE(c->a && c->q && c->d && c->developed && c->expansion, "null crystal array");
  FG_REQUIRE(((reinterpret_cast<uintptr_t>(c->a) | reinterpret_cast<uintptr_t>(c->q) |
               reinterpret_cast<uintptr_t>(c->d)) & 15u) == 0,
             "crystal arrays a, q and d must be 16-byte aligned");
  const bool has64 = c->pos64 != nullptr;
  FG_REQUIRE((c->dims64 != nullptr) == has64 && (c->quat64 != nullptr) == has64,
             "pos64, dims64 and quat64 must be given together or not at all");
  FG_REQUIRE(((reinterpret_cast<uintptr_t>(c->pos64) | reinterpret_cast<uintptr_t>(c->dims64) |
               reinterpret_cast<uintptr_t>(c->quat64) | reinterpret_cast<uintptr_t>(c->expansion)) & 7u) == 0,
             "FP64 arrays pos64, dims64, quat64 and expansion must be 8-byte aligned");
  FG_REQUIRE((reinterpret_cast<uintptr_t>(out) & 3u) == 0, "out must be 4-byte aligned");
  FG_REQUIRE(film->width > 0 && film->height > 0, "film dimensions must be positive");
  FG_REQUIRE(cfg->width_px > 0 && cfg->height_px > 0, "scan size must be positive");
  const uint32_t spp_req = std::max<uint32_t>(cfg->samples_per_pixel, 1);
  const uint32_t g = static_cast<uint32_t>(std::lround(std::sqrt(static_cast<double>(spp_req))));
  const uint32_t a = std::max<uint32_t>(g * g, 1);
  FG_REQUIRE(a <= SCAN_THREADS, "samples_per_pixel too large (at most 256 strata)");

  ScanTile t{};
  t.a = reinterpret_cast<const float4*>(c->a);
  t.q = reinterpret_cast<const float4*>(c->q);
  t.d = reinterpret_cast<const float4*>(c->d);
  t.pos64 = c->pos64;
  t.dims64 = c->dims64;
  t.quat64 = c->quat64;
  t.developed = c->developed;
  t.exp64 = c->expansion;
  t.sigma_c = nullptr;
  t.out = out;
  t.image8 = image8;
  t.d_neg = nullptr;
  t.ray_hits = nullptr;
  t.pw = film->width / static_cast<double>(cfg->width_px);
  t.ph = film->height / static_cast<double>(cfg->height_px);
  t.z0 = film->depth + 0.1;
  t.seed = seed;
  t.bin_base = 0;
  t.w = cfg->width_px;
  t.h = cfg->height_px;
  t.g = g;
  t.spp = a;
  t.bin_px = scan_bin_px(a);
  t.nbx = (t.w + t.bin_px - 1) / t.bin_px;
  t.nby = (t.h + t.bin_px - 1) / t.bin_px;
  t.n = static_cast<uint32_t>(c->n);
  t.sigma = static_cast<float>(cfg->silver_opacity);
  t.mode = cfg->mode;
  t.items_cap = FG_STATIC_SCAN_MAX_ITEMS;
  set_jitter_units(t);
  const unsigned long long nbins = static_cast<unsigned long long>(t.nbx) * t.nby;
  if (nbins > FG_STATIC_SCAN_MAX_BINS)
    throw Error{FG_ERR_INVALID_ARG, "scan of " + std::to_string(t.w) + "x" + std::to_string(t.h) + " px needs " +
                                        std::to_string(nbins) + " bins of " + std::to_string(t.bin_px) +
                                        " px; the static scratch holds at most " +
                                        std::to_string(FG_STATIC_SCAN_MAX_BINS)};

  const int dev = current_device();
  std::lock_guard<std::mutex> call_lock(g_call_mu[dev]);
  unsigned char* base = scratch_for_device(dev);
  auto* desc = reinterpret_cast<ScanTile*>(base + kDescOff);
  auto* err = reinterpret_cast<uint32_t*>(base + kErrOff);
  auto* cnt = reinterpret_cast<uint32_t*>(base + kCntOff);
  auto* off = reinterpret_cast<uint32_t*>(base + kOffOff);
  auto* cur = reinterpret_cast<uint32_t*>(base + kCurOff);
  auto* items = reinterpret_cast<uint32_t*>(base + kItemsOff);
  auto* devlist = reinterpret_cast<uint32_t*>(base + kDevListOff);
  auto* devcount = reinterpret_cast<uint32_t*>(base + kDevCountOff);
  t.bin_off = off;
  t.bin_items = items;

  (void)cudaGetLastError();  // a stale launch error of the caller's is not ours to report
  // From here on work is queued on the scratch: a failure waits for it before the lock is released.
  struct DrainOnThrow {
    cudaStream_t st;
    bool armed = true;
    ~DrainOnThrow() {
      if (armed) (void)cudaStreamSynchronize(st);
    }
  } drain{st};
  // What must start at zero: counts (and the total slot), cursors, the error word, the developed count.
  FG_CUDA(cudaMemsetAsync(cnt, 0, (nbins + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(cur, 0, (nbins + 1) * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(err, 0, 4 * sizeof(uint32_t), st));
  FG_CUDA(cudaMemsetAsync(devcount, 0, sizeof(uint32_t), st));
  // The scan's tree over the developed crystals (transmittance.rs:86-89).
  if (t.n)
    k_static_devlist<<<grid_for(t.n, 256), 256, 0, st>>>(c->developed, t.n, devlist, devcount,
                                                          FG_STATIC_SCAN_MAX_DEVELOPED);
  FG_CUDA(cudaGetLastError());
  uint32_t ndev = 0;
  FG_CUDA(cudaMemcpyAsync(&ndev, devcount, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  if (ndev > FG_STATIC_SCAN_MAX_DEVELOPED)
    throw Error{FG_ERR_INVALID_ARG, std::to_string(ndev) + " developed crystals; the static scratch holds at most " +
                                        std::to_string(FG_STATIC_SCAN_MAX_DEVELOPED)};
  RTreeBufs tree;
  {
    RTile rt{};
    rt.a = t.a;
    rt.d = t.d;
    rt.pos64 = t.pos64;
    rt.dims64 = t.dims64;
    rt.exp64 = t.exp64;
    rt.order = devlist;
    rt.ecap = FG_STATIC_SCAN_MAX_DEVELOPED;
    rt.n = ndev;
    rt.pad = static_cast<float>(std::max(film->width, film->height) * 2e-6 + 1e-5);
    rtree_attach(tree, rt, true, FG_STATIC_SCAN_MAX_CRYSTALS, base + kTreeOff, kTreeBytes, st);
    rtree_build(tree, err, st);
  }
  t.lbox64 = tree.box64.p;
  t.leafof = tree.leafof.p;
  if (t.n) k_bin_count<<<grid_for(t.n, 256), 256, 0, st>>>(t, cnt);
  k_exclusive_scan_small<<<1, kScanThreads, 0, st>>>(cnt, off, static_cast<uint32_t>(nbins + 1));
  FG_CUDA(cudaGetLastError());
  uint32_t total = 0;
  FG_CUDA(cudaMemcpyAsync(&total, off + nbins, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  if (total > FG_STATIC_SCAN_MAX_ITEMS)
    throw Error{FG_ERR_INVALID_ARG, "the developed crystals make " + std::to_string(total) +
                                        " bin entries; the static scratch holds at most " +
                                        std::to_string(FG_STATIC_SCAN_MAX_ITEMS)};
  if (t.n) k_bin_fill<<<grid_for(t.n, 256), 256, 0, st>>>(t, off, cur, items);
  FG_CUDA(cudaGetLastError());
  // The descriptor is copied from this stack frame before the call returns (pageable source).
  FG_CUDA(cudaMemcpyAsync(desc, &t, sizeof(ScanTile), cudaMemcpyHostToDevice, st));
  const unsigned threads = ((t.bin_px * t.bin_px * a + 31) / 32) * 32;  // whole warps
  launch_scan(desc, 1, nbins, threads, err, nullptr, st);
  uint32_t w = 0;
  FG_CUDA(cudaMemcpyAsync(&w, err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  FG_CUDA(cudaStreamSynchronize(st));
  drain.armed = false;  // the stream is drained
  if (w) {
    char hex[16];
    std::snprintf(hex, sizeof(hex), "%08x", w);
    throw Error{FG_ERR_DEVICE_OVERFLOW, std::string("scan kernel error word 0x") + hex};
  }
}

}  // namespace
}  // namespace fg

extern "C" fg_status fg_scan_crystals_static(const fg_device_crystals* crystals, const fg_emulsion_cfg* film,
                                             const fg_scan_cfg* cfg, uint64_t seed, float* out, uint8_t* image8,
                                             void* stream, char* message, size_t message_len) {
  fg::write_message(message, message_len, "");
  try {
    fg::static_scan(crystals, film, cfg, seed, out, image8, static_cast<cudaStream_t>(stream));
    return FG_OK;
  } catch (const fg::Error& e) {
    fg::write_message(message, message_len, e.msg);
    return e.st;
  } catch (const std::exception& e) {
    fg::write_message(message, message_len, e.what());
    return FG_ERR_PIPELINE;
  }
}
