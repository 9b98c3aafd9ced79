// Morton ordering of an uploaded crystal set: crystals live in Morton order on the device (the
// batched path's synthesis emits them in brick order), with the id <-> slot maps.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "fg_internal.h"

namespace fg {

__device__ __forceinline__ uint64_t spread21(uint64_t x) {
  x &= 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ uint64_t morton63(double x, double y, double z, double lx, double ly,
                                             double lz, double inv_ext) {
  auto q = [&](double v, double lo) {
    double t = (v - lo) * inv_ext * 2097152.0;
    t = fmin(fmax(t, 0.0), 2097151.0);
    return static_cast<uint64_t>(t);
  };
  return (spread21(q(x, lx)) << 2) | (spread21(q(y, ly)) << 1) | spread21(q(z, lz));
}

__global__ void k_morton(const double* pos, uint32_t n, double lx, double ly, double lz,
                         double inv_ext, uint64_t* keys, uint32_t* vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  keys[i] = morton63(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], lx, ly, lz, inv_ext);
  vals[i] = i;
}

__global__ void k_gather(const uint32_t* order, uint32_t n, const double* pos, const double* dims,
                         const double* quat, const double* sens, const int32_t* morph,
                         int32_t morph_all, float4* a, float4* q, float4* d, double* pos64,
                         double* dims64, double* quat64, double* sens64, uint32_t* s2id,
                         uint32_t* id2s) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = order[s];
  s2id[s] = i;
  id2s[i] = s;
  const int mo = morph ? morph[i] : morph_all;
  a[s] = make_float4((float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2], (float)sens[i]);
  q[s] = make_float4((float)quat[4 * i], (float)quat[4 * i + 1], (float)quat[4 * i + 2], (float)quat[4 * i + 3]);
  d[s] = make_float4((float)dims[3 * i], (float)dims[3 * i + 1], (float)dims[3 * i + 2], __int_as_float(mo));
  for (int j = 0; j < 3; ++j) {
    pos64[3 * s + j] = pos[3 * i + j];
    dims64[3 * s + j] = dims[3 * i + j];
  }
  for (int j = 0; j < 4; ++j) quat64[4 * s + j] = quat[4 * i + j];
  sens64[s] = sens[i];
}

__device__ __forceinline__ int kdelta(const uint64_t* keys, long long n, long long i, long long j) {
  if (j < 0 || j >= n) return -1;
  const uint64_t ki = keys[i], kj = keys[j];
  if (ki == kj) return 64 + __clz(static_cast<uint32_t>(i ^ j));
  return __clzll(ki ^ kj);
}

void morton_order(fg_emulsion* em, const double* pos_host, const double* pos_dev, cudaStream_t st,
                  DBuf<uint64_t>& keys, DBuf<uint32_t>& order) {
  const uint32_t n = em->n;
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (uint32_t i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) {
      lo[j] = std::min(lo[j], pos_host[3 * i + j]);
      hi[j] = std::max(hi[j], pos_host[3 * i + j]);
    }
  double ext = std::max(std::max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
  if (!(ext > 0.0)) ext = 1.0;
  DBuf<uint64_t> k0(n, st);
  DBuf<uint32_t> v0(n, st);
  keys.alloc(n, st);
  order.alloc(n, st);
  k_morton<<<grid_for(n, 256), 256, 0, st>>>(pos_dev, n, lo[0], lo[1], lo[2], 1.0 / ext, k0.p, v0.p);
  FG_CUDA(cudaGetLastError());
  size_t tmp_bytes = 0;
  FG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k0.p, keys.p, v0.p, order.p, (int)n, 0, 63, st));
  DBuf<unsigned char> tmp(tmp_bytes, st);
  FG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, k0.p, keys.p, v0.p, order.p, (int)n, 0, 63, st));
}

void exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t st) {
  size_t tmp_bytes = 0;
  FG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, in, out, (int)n, st));
  DBuf<unsigned char> tmp(tmp_bytes, st);
  FG_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, in, out, (int)n, st));
}

// Gathers an uploaded (id-ordered, FP64) crystal set into Morton order.  Exposed to the engine
// translation unit through this wrapper.
void gather_sorted(fg_emulsion* em, const uint32_t* order, const double* pos, const double* dims,
                   const double* quat, const double* sens, const int32_t* morph, int32_t morph_all,
                   cudaStream_t st) {
  const uint32_t n = em->n;
  k_gather<<<grid_for(n, 256), 256, 0, st>>>(order, n, pos, dims, quat, sens, morph, morph_all,
                                             em->a.p, em->q.p, em->d.p, em->pos64.p, em->dims64.p,
                                             em->quat64.p, em->sens64.p, em->sorted_to_id.p,
                                             em->id_to_sorted.p);
  FG_CUDA(cudaGetLastError());
}

}  // namespace fg
