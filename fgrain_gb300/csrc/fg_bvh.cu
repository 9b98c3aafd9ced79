// Morton ordering and LBVH construction (Karras, "Maximizing parallelism in the construction of
// BVHs, octrees, and k-d trees", HPG 2012), replacing the reference's sequential spatial-median
// build (bvh.rs:157-295).  Crystals live in Morton order; every internal node stores the boxes of
// both children so a traversal step is one 64-byte node load.
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

// One thread per internal node (Karras 2012, figure 4).
__global__ void k_karras(const uint64_t* keys, uint32_t n, Node* nodes, int* leaf_parent) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)n - 1) return;
  const int dir = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(keys, n, i, i - dir);
  long long lmax = 2;
  while (kdelta(keys, n, i, i + lmax * dir) > dmin) lmax <<= 1;
  long long l = 0;
  for (long long t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(keys, n, i, i + (l + t) * dir) > dmin) l += t;
  const long long j = i + l * dir;
  const int dnode = kdelta(keys, n, i, j);
  long long s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(keys, n, i, i + (s + t) * dir) > dnode) s += t;
  } while (t > 1);
  const long long gamma = i + s * dir + (dir < 0 ? -1 : 0);
  const long long lo = i < j ? i : j, hi = i < j ? j : i;
  int left, right;
  if (lo == gamma) {
    left = ~static_cast<int>(gamma);
    leaf_parent[gamma] = static_cast<int>(i);
  } else {
    left = static_cast<int>(gamma);
    nodes[gamma].d.z = static_cast<int>(i);
  }
  if (hi == gamma + 1) {
    right = ~static_cast<int>(gamma + 1);
    leaf_parent[gamma + 1] = static_cast<int>(i);
  } else {
    right = static_cast<int>(gamma + 1);
    nodes[gamma + 1].d.z = static_cast<int>(i);
  }
  nodes[i].d.x = left;
  nodes[i].d.y = right;
  nodes[i].d.w = static_cast<int>(hi);
  if (i == 0) nodes[0].d.z = -1;
}

// Leaf box: the bounding box of the crystal shape (oriented cube or ellipsoid), padded outward by
// pad.  It is not cut by the crystal's own max_dim box: a canonical hit tests that box on the
// whole ray, while its entry distance is the shape's, so culling by entry distance needs the
// full shape.  An empty box is NaN (never hit: every comparison with NaN is false).
__device__ __forceinline__ void leaf_box(const float4 a, const float4 q, const float4 d, float e,
                                         float pad, float* lo, float* hi) {
  const float x = q.x, y = q.y, z = q.z, w = q.w;
  const float R[3][3] = {{1.f - 2.f * (y * y + z * z), 2.f * (x * y - z * w), 2.f * (x * z + y * w)},
                         {2.f * (x * y + z * w), 1.f - 2.f * (x * x + z * z), 2.f * (y * z - x * w)},
                         {2.f * (x * z - y * w), 2.f * (y * z + x * w), 1.f - 2.f * (x * x + y * y)}};
  const float dm[3] = {d.x * e, d.y * e, d.z * e};
  const bool cubic = __float_as_int(d.w) == 0;
  const float p[3] = {a.x, a.y, a.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float ext;
    if (cubic) {
      ext = fabsf(R[i][0]) * dm[0] + fabsf(R[i][1]) * dm[1] + fabsf(R[i][2]) * dm[2];
    } else {
      const float u = R[i][0] * dm[0], v = R[i][1] * dm[1], t = R[i][2] * dm[2];
      ext = sqrtf(u * u + v * v + t * t);
    }
    const float h = ext * 1.0001f + pad;
    lo[i] = p[i] - h;
    hi[i] = p[i] + h;
  }
}

__device__ __forceinline__ void store_slot(Node* nodes, int parent, int code, const float* lo,
                                           const float* hi) {
  float* f = reinterpret_cast<float*>(&nodes[parent]);
  const int off = (nodes[parent].d.x == code) ? 0 : 6;
  __stcg(f + off + 0, lo[0]);
  __stcg(f + off + 1, lo[1]);
  __stcg(f + off + 2, lo[2]);
  __stcg(f + off + 3, hi[0]);
  __stcg(f + off + 4, hi[1]);
  __stcg(f + off + 5, hi[2]);
}

// Bottom-up box fit: the second thread to reach a node unites its children and climbs on.
__global__ void k_fit(const float4* A, const float4* Q, const float4* D, const uint8_t* developed,
                      const float* exp32, uint32_t n, Node* nodes, const int* leaf_parent,
                      int* visit, float pad, int developed_geometry) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float lo[3], hi[3];
  if (developed_geometry && !developed[s]) {
    lo[0] = lo[1] = lo[2] = hi[0] = hi[1] = hi[2] = __int_as_float(0x7fc00000);
  } else {
    const float e = developed_geometry ? exp32[s] : 1.0f;
    leaf_box(A[s], Q[s], D[s], e, pad, lo, hi);
  }
  int code = ~static_cast<int>(s);
  int p = leaf_parent[s];
  while (p >= 0) {
    store_slot(nodes, p, code, lo, hi);
    __threadfence();
    if (atomicAdd(&visit[p], 1) == 0) return;
    __threadfence();
    const float* f = reinterpret_cast<const float*>(&nodes[p]);
    float v[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = __ldcg(f + k);
    lo[0] = fminf(v[0], v[6]);
    lo[1] = fminf(v[1], v[7]);
    lo[2] = fminf(v[2], v[8]);
    hi[0] = fmaxf(v[3], v[9]);
    hi[1] = fmaxf(v[4], v[10]);
    hi[2] = fmaxf(v[5], v[11]);
    code = p;
    p = __ldcg(&nodes[p].d.z);
  }
}

// Outward padding of leaf boxes: covers rounding of FP64 positions and of FP64 rays to FP32.
static float leaf_pad(const fg_emulsion* em) {
  const double ext = std::max(em->extent, std::max(std::max(std::fabs(em->cfg.width),
                                                            std::fabs(em->cfg.height)),
                                                   std::fabs(em->cfg.depth)));
  return static_cast<float>(ext * 2e-6 + 1e-5);
}

void refit_lbvh(fg_emulsion* em, Node* nodes, const int* leaf_parent, bool developed_geometry,
                cudaStream_t st) {
  const uint32_t n = em->n;
  if (n == 0) return;
  DBuf<int> visit(std::max<uint32_t>(n - 1, 1), st);
  FG_CUDA(cudaMemsetAsync(visit.p, 0, visit.n * sizeof(int), st));
  if (n == 1) {
    // A lone crystal hangs off a root whose second child is empty.
    const int one = 1;
    FG_CUDA(cudaMemcpyAsync(visit.p, &one, sizeof(int), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaStreamSynchronize(st));
  }
  k_fit<<<grid_for(n, 256), 256, 0, st>>>(em->a.p, em->q.p, em->d.p, em->developed.p, em->exp32.p,
                                          n, nodes, leaf_parent, visit.p, leaf_pad(em),
                                          developed_geometry ? 1 : 0);
  FG_CUDA(cudaGetLastError());
}

void build_lbvh(fg_emulsion* em, const uint64_t* keys, Node* nodes, int* leaf_parent,
                bool developed_geometry, cudaStream_t st) {
  const uint32_t n = em->n;
  if (n == 0) return;
  if (n == 1) {
    Node root;
    const float nanf_ = std::nanf("");
    root.a = make_float4(nanf_, nanf_, nanf_, nanf_);
    root.b = make_float4(nanf_, nanf_, nanf_, nanf_);
    root.c = make_float4(nanf_, nanf_, nanf_, nanf_);
    root.d = make_int4(~0, INT32_MIN, -1, 0);
    const int zero = 0;
    FG_CUDA(cudaMemcpyAsync(nodes, &root, sizeof(Node), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaMemcpyAsync(leaf_parent, &zero, sizeof(int), cudaMemcpyHostToDevice, st));
    FG_CUDA(cudaStreamSynchronize(st));
  } else {
    k_karras<<<grid_for(n - 1, 256), 256, 0, st>>>(keys, n, nodes, leaf_parent);
    FG_CUDA(cudaGetLastError());
  }
  refit_lbvh(em, nodes, leaf_parent, developed_geometry, st);
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
