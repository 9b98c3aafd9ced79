// Device builder of the reference tree (BVH::build / subdivide, bvh.rs:157-295); see fg_rtree.cuh.
//
// The tree's topology is built top-down, one level at a time over all tiles of a batch:
//   reduce  each pending node's centroid box (min / max on order-preserving 64-bit keys of the
//           FP64 values: exact whatever the order, and on the integer pipes);
//   decide  leaf or split (largest centroid extent, midpoint 0.5 (lo + hi)), children ids;
//   flag    every element of a splitting node: centroid >= mid ("big"), with the prefix sum of the
//           flags (ranks of bigs inside each node's contiguous range) in the same passes;
//   pq      P_m = position of the m-th big from the left, Q_m = of the m-th small from the right;
//   place   every element moves to where the reference's swap partition puts it (below).
// The splits read only the centroids (bvh.rs:196-258), so each element's three order-preserving
// 64-bit centroid keys (of its FP64 max_dim box, computed once) travel with it, and every pass
// reads them in order and does no FP64 work.  Nodes of at most RT_CTA_MAX elements leave the
// global levels: one thread block each builds their subtree with the elements in shared memory,
// the same passes per level, all levels down to the leaves.  Centroid boxes are reduced
// segment-wise (a node is a contiguous range of positions).  The node boxes (the union of the
// elements' boxes, which the reference stores but never splits on) are formed bottom up: a block
// forms those of its subtree after its last level, k_rt_refit those above the blocks' subtrees;
// min and max are exact, so the order does not matter.
//
// The swap partition (bvh.rs:244-258: i from the left, j from the right; a small at i stays and i
// advances, a big at i is swapped with j and j retreats) examines the range as two streams: the
// left stream runs while it sees smalls, the right stream while it sees bigs.  With S the number
// of smalls, K = the number of bigs among the first S positions (the pairs the swaps exchange) and
// Q_0 = n, the left stream covers [0, li) where li = S + 1 if position S holds a big, else S; and
// the element at relative position r goes to
//   r < li, small:            r                      (stays)
//   r < li, the m-th big:     Q_{m-1} - 1            (bigs fill the right end in examination order)
//   r >= li, the m-th small from the right:  P_m     (takes the place of the m-th big)
//   r >= li, big:             r - 1                  (shifts one place towards the middle)
// S is the left child's size.  A simulation of the reference loop confirms the rule and the closed
// forms of K and li on random ranges.
#include <algorithm>
#include <climits>
#include <cmath>
#include <type_traits>

#include "fg_internal.h"
#include "fg_rtree.cuh"

namespace fg {

namespace {

constexpr unsigned RT_BLOCK = 256;

// Global split levels for trees of up to emax elements: halving down to the per-block size, plus a
// wide margin for uneven splits (unused levels cost only launches that find no work).
int levels_for(uint32_t emax) {
  if (emax <= static_cast<uint32_t>(RT_CTA_MAX)) return 0;
  int lv = 0;
  while ((static_cast<unsigned long long>(RT_CTA_MAX) << lv) < emax) ++lv;
  return std::min(lv + 8, 44);
}

constexpr unsigned SCAN_ITEMS = 2048;  // entries per block of the prefix sum (256 threads x 8)

__device__ __forceinline__ unsigned long long ord64(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unord64(unsigned long long u) {
  const unsigned long long b = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
  return __longlong_as_double(static_cast<long long>(b));
}

__device__ __forceinline__ int rt_tile_of(const RTile* tiles, int ntiles, unsigned long long x) {
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].ebase <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct RtArgs {
  RTile* tiles;
  int ntiles;
  unsigned long long E, N;
  uint32_t* idx[2];
  // Keys of the element at position x, field f at key[c][f * E + x]: ord64 of the centroid xyz.
  unsigned long long* key[2];
  uint32_t* nof[2];
  uint32_t* flag;
  uint32_t* bb;
  uint32_t* blk;
  uint32_t* P;
  uint32_t* Q;
  uint32_t* ridx;
  unsigned long long* acc;
  double* box64;
  uint32_t* parent;  // parent id of each node (RT_NONE for a root)
  uint32_t *nstart, *ncount, *ntile, *ndepth;
  int* nsplit;
  double* nmid;
  int2* nchild;
  uint32_t* wl[2];
  uint32_t* bq;     // block queue: nodes of at most RT_CTA_MAX elements
  uint32_t* bqpar;  // and the buffer parity holding their elements
  uint32_t* cnt;    // [0], [1] worklist counts, [2] block queue count
  uint32_t* err;
};

// Node allocation: two tile-local ids, or none when the tile's node capacity is spent.
__device__ __forceinline__ bool alloc_pair(const RtArgs& A, int t, uint32_t& l) {
  l = atomicAdd(&A.tiles[t].nodes, 2u);
  if (l + 2 > A.tiles[t].ncap) {
    atomicOr(A.err, ERR_LIST_OVERFLOW);
    return false;
  }
  return true;
}

constexpr uint32_t RT_NONE = 0xffffffffu;
constexpr uint32_t RT_BOX_ONLY = 2;  // block-queue entry of a finished leaf: only its box is formed

// Hands a new node of n elements (held in buffer `par`) to the phase that builds it: the global
// levels (more than RT_CTA_MAX elements; its centroid accumulators start empty) or one block.
__device__ __forceinline__ void rt_enqueue(const RtArgs& A, uint32_t id, uint32_t n, int par) {
  A.nsplit[id] = -1;
  if (n > static_cast<uint32_t>(RT_CTA_MAX)) {
    unsigned long long* a = A.acc + 6ull * id;
#pragma unroll
    for (int k = 0; k < 3; ++k) a[k] = ~0ull;  // minima
#pragma unroll
    for (int k = 3; k < 6; ++k) a[k] = 0ull;  // maxima
    A.wl[par][atomicAdd(&A.cnt[par], 1u)] = id;
  } else if (n > 0) {
    const uint32_t q = atomicAdd(&A.cnt[2], 1u);
    A.bq[q] = id;
    A.bqpar[q] = static_cast<uint32_t>(par);
  }
}

// The 6 reduction keys of the element at position x of a key array (field f at key[f * stride +
// x]): centroid xyz as minima, then as maxima.  Min and max are exact in any order, and on the
// ordered 64-bit keys they run on the integer pipes (GB300's FP64 pipe is narrow).
__device__ __forceinline__ void rt_keys(const unsigned long long* key, unsigned long long stride, unsigned long long x,
                                        unsigned long long k[6]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    k[i] = key[i * stride + x];
    k[3 + i] = k[i];
  }
}

// The three centroid keys of element slot s of tile T, written to position x of key[f * stride +
// x] (normalised so that -0 orders as +0, as the FP64 comparisons see them).
__device__ __forceinline__ void rt_key3(const RTile& T, uint32_t s, unsigned long long* key, unsigned long long stride,
                                        unsigned long long x) {
  double lo[3], hi[3], cc[3];
  rt_box_pm(rt_pm(T, s), lo, hi, cc);
#pragma unroll
  for (int i = 0; i < 3; ++i) key[i * stride + x] = ord64(__dadd_rn(cc[i], 0.0));
}

// Element order and roots.  Thread x < E fills position x; one thread per tile sets up its root.
__global__ void k_rt_init(RtArgs A) {
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  const unsigned long long g0 = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
  for (unsigned long long x = g0; x < A.E; x += stride) {
    const int t = rt_tile_of(A.tiles, A.ntiles, x);
    const RTile& T = A.tiles[t];
    const unsigned long long k = x - T.ebase;
    uint32_t v = RT_DONE;
    if (k < T.n) {
      const uint32_t slot = T.order ? static_cast<uint32_t>(T.order[k] - T.obase) : static_cast<uint32_t>(k);
      A.idx[0][x] = slot;
      rt_key3(T, slot, A.key[0], A.E, x);
      v = T.n > static_cast<uint32_t>(RT_CTA_MAX) ? static_cast<uint32_t>(T.nbase + 1) : RT_DONE;
    }
    A.nof[0][x] = v;
  }
  for (unsigned long long t = g0; t < static_cast<unsigned long long>(A.ntiles); t += stride) {
    RTile& T = A.tiles[t];
    T.nodes = 2;
    T.depth = T.n ? 1 : 0;
    const unsigned long long root = T.nbase + 1;
    A.nstart[root] = static_cast<uint32_t>(T.ebase);
    A.ncount[root] = T.n;
    A.ntile[root] = static_cast<uint32_t>(t);
    A.ndepth[root] = 1;
    A.parent[root] = RT_NONE;
    rt_enqueue(A, static_cast<uint32_t>(root), T.n, 0);
  }
}

__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) { return a < b ? a : b; }
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// Segment-wise reduction over a warp's 32 consecutive positions: lanes with equal `seg` form
// contiguous runs (a node is a contiguous range of positions, so equal values at two lanes mean
// the same node in between).  On return the first lane of each run holds the run's minima
// (k[0..2]) and maxima (k[3..5]); the return value says whether this lane is a run's first.
// Lanes without a node pass a seg value no other lane has.  All 32 lanes call it.
__device__ __forceinline__ bool rt_seg_reduce(uint32_t seg, unsigned long long k[6]) {
  const int lane = threadIdx.x & 31;
  if (__all_sync(0xffffffffu, __shfl_sync(0xffffffffu, seg, 0) == seg)) {
    // One node across the warp (the common case): each 64-bit minimum or maximum as two 32-bit
    // warp reductions, the high words, then the low words of the lanes holding that high word.
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const uint32_t hi = static_cast<uint32_t>(k[i] >> 32), lo = static_cast<uint32_t>(k[i]);
      uint32_t h, l;
      if (i < 3) {
        h = __reduce_min_sync(0xffffffffu, hi);
        l = __reduce_min_sync(0xffffffffu, hi == h ? lo : 0xffffffffu);
      } else {
        h = __reduce_max_sync(0xffffffffu, hi);
        l = __reduce_max_sync(0xffffffffu, hi == h ? lo : 0u);
      }
      k[i] = (static_cast<unsigned long long>(h) << 32) | l;
    }
    return lane == 0;
  }
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t ns = __shfl_down_sync(0xffffffffu, seg, o);
    const bool take = lane + o < 32 && ns == seg;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const unsigned long long y = __shfl_down_sync(0xffffffffu, k[i], o);
      if (take) k[i] = i < 3 ? umin64(k[i], y) : umax64(k[i], y);
    }
  }
  const uint32_t up = __shfl_up_sync(0xffffffffu, seg, 1);
  return lane == 0 || up != seg;
}

__device__ __forceinline__ void rt_keys_empty(unsigned long long k[6]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    k[i] = ~0ull;
    k[3 + i] = 0ull;
  }
}

// Centroid box of every pending node: segment-wise per warp, then one set of 6 atomics per warp
// and node.
__global__ void k_rt_reduce(RtArgs A, int c) {
  if (A.cnt[c] == 0) return;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long base = blockIdx.x * static_cast<unsigned long long>(blockDim.x); base < A.E; base += stride) {
    const unsigned long long x = base + threadIdx.x;
    const uint32_t node = x < A.E ? A.nof[c][x] : RT_DONE;
    const bool act = !(node & RT_DONE);
    if (!__any_sync(0xffffffffu, act)) continue;
    unsigned long long k[6];
    if (act) rt_keys(A.key[c], A.E, x, k); else rt_keys_empty(k);
    const bool head = rt_seg_reduce(act ? node : (RT_DONE | (threadIdx.x & 31)), k);
    if (act && head) {
      unsigned long long* a = A.acc + 6ull * node;
#pragma unroll
      for (int i = 0; i < 3; ++i) atomicMin(a + i, k[i]);
#pragma unroll
      for (int i = 3; i < 6; ++i) atomicMax(a + i, k[i]);
    }
  }
}

// Leaf or split for every pending node of this level (subdivide, bvh.rs:200-270).
__global__ void k_rt_decide(RtArgs A, int c) {
  const uint32_t nw = A.cnt[c];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) {
    const uint32_t node = A.wl[c][i];
    const int t = static_cast<int>(A.ntile[node]);
    const unsigned long long* a = A.acc + 6ull * node;
    double clo[3], chi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      clo[k] = unord64(a[k]);
      chi[k] = unord64(a[3 + k]);
    }
    const double ex = __dsub_rn(chi[0], clo[0]), ey = __dsub_rn(chi[1], clo[1]), ez = __dsub_rn(chi[2], clo[2]);
    const int axis = (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
    const double ext = axis == 0 ? ex : (axis == 1 ? ey : ez);
    uint32_t l = 0;
    if (A.ncount[node] <= 4 || ext <= 1e-7 || !alloc_pair(A, t, l)) {
      A.nsplit[node] = -1;  // leaf (degenerate centroids, or no node capacity left)
      const uint32_t q = atomicAdd(&A.cnt[2], 1u);  // a block forms its box
      A.bq[q] = node;
      A.bqpar[q] = RT_BOX_ONLY;
      continue;
    }
    A.nsplit[node] = axis;
    A.nmid[node] = __dmul_rn(0.5, __dadd_rn(clo[axis], chi[axis]));
    const unsigned long long nb = A.tiles[t].nbase;
    A.nchild[node] = make_int2(static_cast<int>(nb + l), static_cast<int>(nb + l + 1));
    A.parent[nb + l] = node;
    A.parent[nb + l + 1] = node;
  }
}

// Exclusive prefix sum of flag[0..E] into bb, in blocks of SCAN_ITEMS: block sums, one block
// scanning the block sums, then each block's own scan.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* sh, uint32_t& total) {
  const unsigned lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= static_cast<unsigned>(o)) incl += y;
  }
  if (lane == 31) sh[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t s = lane < blockDim.x / 32 ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= static_cast<unsigned>(o)) s += y;
    }
    sh[lane] = s;
  }
  __syncthreads();
  total = sh[blockDim.x / 32 - 1];
  const uint32_t r = incl - v + (w ? sh[w - 1] : 0u);
  __syncthreads();
  return r;
}

// The flag of position x: its element's centroid >= the split of its node ("big"), 0 when the
// node does not split (or x is done or past the end).
__device__ __forceinline__ uint32_t rt_flag(const RtArgs& A, int c, unsigned long long x) {
  if (x >= A.E) return 0u;
  const uint32_t node = A.nof[c][x];
  if (node & RT_DONE) return 0u;
  const int axis = A.nsplit[node];
  if (axis < 0) return 0u;
  return A.key[c][axis * A.E + x] < ord64(A.nmid[node]) ? 0u : 1u;
}

// Flags and their block sums.
__global__ void __launch_bounds__(RT_BLOCK) k_rt_scan_blocks(RtArgs A, int c, unsigned long long nb) {
  if (A.cnt[c] == 0) return;
  __shared__ uint32_t sh[32];
  for (unsigned long long b = blockIdx.x; b < nb; b += gridDim.x) {
    const unsigned long long x0 = b * SCAN_ITEMS + threadIdx.x * 8ull;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (x0 + k <= A.E) {
        const uint32_t f = rt_flag(A, c, x0 + k);
        A.flag[x0 + k] = f;
        s += f;
      }
    uint32_t tot;
    block_excl_scan(s, sh, tot);
    if (threadIdx.x == 0) A.blk[b] = tot;
  }
}

__global__ void __launch_bounds__(1024) k_rt_scan_top(RtArgs A, int c, unsigned long long nb) {
  if (A.cnt[c] == 0) return;
  __shared__ uint32_t sh[32];
  uint32_t carry = 0;
  for (unsigned long long base = 0; base < nb; base += 1024) {
    const unsigned long long i = base + threadIdx.x;
    const uint32_t v = i < nb ? A.blk[i] : 0u;
    uint32_t tot;
    const uint32_t e = block_excl_scan(v, sh, tot);
    if (i < nb) A.blk[i] = carry + e;
    carry += tot;
  }
}

__global__ void __launch_bounds__(RT_BLOCK) k_rt_scan_final(RtArgs A, int c, unsigned long long nb) {
  if (A.cnt[c] == 0) return;
  __shared__ uint32_t sh[32];
  for (unsigned long long b = blockIdx.x; b < nb; b += gridDim.x) {
    const unsigned long long x0 = b * SCAN_ITEMS + threadIdx.x * 8ull;
    uint32_t f[8], s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      f[k] = x0 + k <= A.E ? A.flag[x0 + k] : 0u;
      s += f[k];
    }
    uint32_t tot;
    uint32_t acc = A.blk[b] + block_excl_scan(s, sh, tot);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (x0 + k <= A.E) {
        A.bb[x0 + k] = acc;
        acc += f[k];
      }
  }
}

// Ranks: P_m (m-th big from the left) and Q_m (m-th small from the right), relative positions.
__global__ void k_rt_pq(RtArgs A, int c) {
  if (A.cnt[c] == 0) return;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long x = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; x < A.E;
       x += stride) {
    const uint32_t node = A.nof[c][x];
    if ((node & RT_DONE) || A.nsplit[node] < 0) continue;
    const uint32_t s = A.nstart[node], n = A.ncount[node];
    const uint32_t r = static_cast<uint32_t>(x - s);
    const uint32_t bs = A.bb[s];
    const uint32_t Bb = A.bb[x] - bs, Bt = A.bb[s + n] - bs, St = n - Bt;
    if (A.flag[x]) {
      A.P[s + Bb] = r;  // m = Bb + 1
    } else {
      const uint32_t mr = St - (r - Bb);  // right rank, 1-based
      A.Q[s + mr - 1] = r;
    }
  }
}

// Moves every element of a splitting node to its place after the reference's swap partition;
// finishes the elements of new leaves; sets up the children.
__global__ void k_rt_place(RtArgs A, int c) {
  if (A.cnt[c] == 0) return;
  const int o = c ^ 1;
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long x = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; x < A.E;
       x += stride) {
    const uint32_t node = A.nof[c][x];
    if (node & RT_DONE) {
      A.nof[o][x] = RT_DONE;
      continue;
    }
    const uint32_t el = A.idx[c][x];
    if (A.nsplit[node] < 0) {  // a leaf of this level: its order is final
      A.ridx[x] = el;
      A.nof[o][x] = RT_DONE;
      continue;
    }
    const uint32_t s = A.nstart[node], n = A.ncount[node];
    const uint32_t r = static_cast<uint32_t>(x - s);
    const uint32_t bs = A.bb[s];
    const uint32_t Bb = A.bb[x] - bs, Bt = A.bb[s + n] - bs, St = n - Bt;
    const uint32_t li = St + (St < n ? A.flag[s + St] : 0u);
    const bool big = A.flag[x] != 0;
    uint32_t dest;
    if (r < li) {
      dest = big ? ((Bb == 0 ? n : A.Q[s + Bb - 1]) - 1) : r;
    } else {
      dest = big ? r - 1 : A.P[s + (St - (r - Bb)) - 1];
    }
    // The reference splits at count / 2 when every centroid fell on one side (bvh.rs:260-265).
    const uint32_t Sp = (St == 0 || St == n) ? n / 2 : St;
    const int2 ch = A.nchild[node];
    const bool left = dest < Sp;
    const uint32_t child = static_cast<uint32_t>(left ? ch.x : ch.y);
    const uint32_t csize = left ? Sp : n - Sp;
    A.idx[o][s + dest] = el;
#pragma unroll
    for (int f = 0; f < 3; ++f) A.key[o][f * A.E + s + dest] = A.key[c][f * A.E + x];
    A.nof[o][s + dest] = csize > static_cast<uint32_t>(RT_CTA_MAX) ? child : RT_DONE;
    if (r == 0) {
      const uint32_t t = A.ntile[node], dep = A.ndepth[node] + 1;
      const uint32_t cs[2] = {Sp, n - Sp};
      const uint32_t cid[2] = {static_cast<uint32_t>(ch.x), static_cast<uint32_t>(ch.y)};
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const uint32_t id = cid[k];
        A.nstart[id] = s + (k ? Sp : 0u);
        A.ncount[id] = cs[k];
        A.ntile[id] = t;
        A.ndepth[id] = dep;
        rt_enqueue(A, id, cs[k], o);
      }
      atomicMax(&A.tiles[t].depth, dep);
    }
  }
}

__global__ void k_rt_level_end(RtArgs A, int c) {
  // The worklist of this level has been consumed; the next level's count was filled by place.
  A.cnt[c] = 0;
}

__global__ void k_rt_check(RtArgs A, int c) {
  if (A.cnt[c] != 0) atomicOr(A.err, ERR_LIST_OVERFLOW);  // nodes left after the last level
}

// The block queue: one block builds the whole subtree of a node of at most RT_CTA_MAX elements
// with its elements in shared memory.  Each level runs the passes of the global levels over all
// of the level's nodes of more than RT_LEAF_MAX elements at once (segment-wise reduce, decide,
// flags and prefix sum, ranks, place); a child of at most RT_LEAF_MAX elements is a leaf
// (bvh.rs:200-204), whose fields one thread writes at the start of the next level.
constexpr int RT_CTA_T = 256;                                // threads per block
constexpr int RT_CTA_PER = RT_CTA_MAX / RT_CTA_T;            // positions per thread
constexpr int RT_LEAF_MAX = 4;                               // subdivide's leaf size
constexpr int RT_CTA_LV = RT_CTA_MAX / (RT_LEAF_MAX + 1);    // nodes of more than 4 per level (204)
constexpr int RT_CTA_SL = 2 * RT_CTA_LV;                     // leaves of at most 4 made by one level
constexpr uint8_t RT_CTA_FREE = 0xff;                        // position of a finished range
constexpr int RT_CTA_LVMAX = RT_MAX_DEPTH + 1;               // levels of a job (deeper trees are rejected)
static_assert(RT_CTA_LV < RT_CTA_FREE, "level slots must fit a byte");
static_assert(RT_CTA_MAX <= 2048, "positions are packed in 11 bits");

struct RtCtaSmem {
  unsigned long long key[3][RT_CTA_MAX];  // the job's centroid keys, at their load position (home)
  // Per level: the nodes' centroid accumulators (reduce to decide), then the flags' prefix sum and
  // the ranks (flags to place); the two uses do not overlap.
  union {
    unsigned long long acc[RT_CTA_LV][6];   // per level node: ordered minima, maxima
    struct {
      uint16_t bb[RT_CTA_MAX + 1];          // exclusive prefix sum of the flags
      uint16_t P[RT_CTA_MAX], Q[RT_CTA_MAX];
    } r;
  } u;
  double mid[RT_CTA_LV];
  uint32_t idx[RT_CTA_MAX];               // element slot
  uint16_t home[RT_CTA_MAX];              // element's load position (its keys)
  uint32_t id[2][RT_CTA_LV];              // this level's nodes and the next's
  uint32_t child[RT_CTA_LV];              // first child id of a splitting node
  uint32_t sl[RT_CTA_SL];                 // small leaves: position | count << 11 | depth << 14
  uint32_t slid[RT_CTA_SL];
  uint32_t scan[RT_CTA_T / 32];
  uint16_t off[2][RT_CTA_LV], cnt[2][RT_CTA_LV];
  uint16_t sp[RT_CTA_LV];                 // left child size
  uint8_t nd[RT_CTA_MAX];                 // level slot of the position's node, RT_CTA_FREE when done
  uint8_t flag[RT_CTA_MAX];
  uint8_t dep[2][RT_CTA_LV];
  uint8_t cslot[RT_CTA_LV][2];            // next-level slot of each child, RT_CTA_FREE for a small leaf
  int8_t axis[RT_CTA_LV];
  int nl, nsl, nnext, nslnew;
  uint32_t maxdep;
  int nint, nlvl;                         // internal nodes of the job so far, and levels
  uint16_t lvend[RT_CTA_LVMAX];           // internal nodes listed after each level
};

// Folds the max_dim box of element slot `slot` into k (minima 0-2, maxima 3-5, ordered keys).
__device__ __forceinline__ void rt_fold_box(const RTile& T, uint32_t slot, unsigned long long k[6]) {
  double lo[3], hi[3], cc[3];
  rt_box_pm(rt_pm(T, slot), lo, hi, cc);
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    k[m] = umin64(k[m], ord64(lo[m]));
    k[3 + m] = umax64(k[3 + m], ord64(hi[m]));
  }
}

__device__ __forceinline__ void rt_store_box(const RtArgs& A, uint32_t id, const unsigned long long k[6]) {
#pragma unroll
  for (int m = 0; m < 6; ++m) A.box64[6ull * id + m] = unord64(k[m]);
}

// Four blocks per SM (64 registers; the block's shared memory is about 53 KB): 9 % faster than two.
__global__ void __launch_bounds__(RT_CTA_T, 4) k_rt_cta(RtArgs A) {
  extern __shared__ __align__(32) unsigned char rt_cta_raw[];
  RtCtaSmem& S = *reinterpret_cast<RtCtaSmem*>(rt_cta_raw);
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const uint32_t nq = A.cnt[2];
  for (uint32_t q = blockIdx.x; q < nq; q += gridDim.x) {
    const uint32_t root = A.bq[q], par = A.bqpar[q];
    const uint32_t s = A.nstart[root];
    if (par == RT_BOX_ONLY) {  // a leaf of the global levels: its box, from all its elements
      const RTile& T = A.tiles[A.ntile[root]];
      const uint32_t cn = A.ncount[root];
      if (tid < 6) S.u.acc[0][tid] = tid < 3 ? ~0ull : 0ull;
      __syncthreads();
      unsigned long long k[6];
      rt_keys_empty(k);
      for (uint32_t j = tid; j < cn; j += RT_CTA_T) rt_fold_box(T, A.ridx[s + j], k);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        atomicMin(&S.u.acc[0][m], k[m]);
        atomicMax(&S.u.acc[0][3 + m], k[3 + m]);
      }
      __syncthreads();
      if (tid == 0) rt_store_box(A, root, S.u.acc[0]);
      __syncthreads();
      continue;
    }
    const int n = static_cast<int>(min(A.ncount[root], static_cast<uint32_t>(RT_CTA_MAX)));
    const uint32_t t = A.ntile[root];
    const unsigned long long nb = A.tiles[t].nbase;
    const uint32_t dep0 = min(A.ndepth[root], 255u);
    for (int x = tid; x < RT_CTA_MAX; x += RT_CTA_T) {
      if (x < n) {
#pragma unroll
        for (int f = 0; f < 3; ++f) S.key[f][x] = A.key[par][f * A.E + s + x];
        S.home[x] = static_cast<uint16_t>(x);
        S.idx[x] = A.idx[par][s + x];
        S.nd[x] = n > RT_LEAF_MAX ? 0 : RT_CTA_FREE;
      } else {
        S.nd[x] = RT_CTA_FREE;
      }
    }
    if (tid == 0) {
      S.maxdep = 0;
      S.nint = 0;
      S.nlvl = 0;
      if (n > RT_LEAF_MAX) {
        S.nl = 1;
        S.nsl = 0;
        S.id[0][0] = root;
        S.off[0][0] = 0;
        S.cnt[0][0] = static_cast<uint16_t>(n);
        S.dep[0][0] = static_cast<uint8_t>(dep0);
      } else {
        S.nl = 0;
        S.nsl = 1;
        S.sl[0] = static_cast<uint32_t>(n) << 11 | dep0 << 14;
        S.slid[0] = root;
      }
    }
    __syncthreads();
    int cur = 0;
    for (;;) {
      const int nl = S.nl, nsl = S.nsl;
      // Leaves of at most four elements made by the previous level (or a small root).
      for (int i = tid; i < nsl; i += RT_CTA_T) {
        const uint32_t e = S.sl[i], id = S.slid[i];
        const int o0 = static_cast<int>(e & 2047u), cn = static_cast<int>((e >> 11) & 7u);
        const uint32_t dp = e >> 14;
        unsigned long long k[6];
        rt_keys_empty(k);
        for (int j = 0; j < cn; ++j) rt_fold_box(A.tiles[t], S.idx[o0 + j], k);
        rt_store_box(A, id, k);
        A.nstart[id] = s + static_cast<uint32_t>(o0);
        A.ncount[id] = static_cast<uint32_t>(cn);
        A.ntile[id] = t;
        A.ndepth[id] = dp;
        A.nsplit[id] = -1;
        atomicMax(&S.maxdep, dp);
      }
      for (int i = tid; i < nl * 6; i += RT_CTA_T) S.u.acc[i / 6][i % 6] = (i % 6) < 3 ? ~0ull : 0ull;
      __syncthreads();
      if (nl == 0) break;
      if (tid == 0) {
        S.nnext = 0;
        S.nslnew = 0;
      }
      // Reduce: position x = k * RT_CTA_T + tid, so a warp holds 32 consecutive positions.
#pragma unroll 1
      for (int k = 0; k < RT_CTA_PER; ++k) {
        const int x = k * RT_CTA_T + tid;
        const uint32_t node = S.nd[x];
        const bool act = node != RT_CTA_FREE;
        if (!__any_sync(0xffffffffu, act)) continue;
        unsigned long long kk[6];
        if (act) rt_keys(&S.key[0][0], RT_CTA_MAX, S.home[x], kk); else rt_keys_empty(kk);
        const bool head = rt_seg_reduce(act ? node : (0x100u | static_cast<uint32_t>(lane)), kk);
        if (act && head) {
#pragma unroll
          for (int i = 0; i < 3; ++i) atomicMin(&S.u.acc[node][i], kk[i]);
#pragma unroll
          for (int i = 3; i < 6; ++i) atomicMax(&S.u.acc[node][i], kk[i]);
        }
      }
      __syncthreads();
      // Decide (subdivide, bvh.rs:200-270), one thread per node of the level.
      for (int i = tid; i < nl; i += RT_CTA_T) {
        const uint32_t id = S.id[cur][i];
        const int cn = S.cnt[cur][i];
        double clo[3], chi[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          clo[m] = unord64(S.u.acc[i][m]);
          chi[m] = unord64(S.u.acc[i][3 + m]);
        }
        A.nstart[id] = s + S.off[cur][i];
        A.ncount[id] = static_cast<uint32_t>(cn);
        A.ntile[id] = t;
        A.ndepth[id] = S.dep[cur][i];
        atomicMax(&S.maxdep, static_cast<uint32_t>(S.dep[cur][i]));
        const double ex = __dsub_rn(chi[0], clo[0]), ey = __dsub_rn(chi[1], clo[1]), ez = __dsub_rn(chi[2], clo[2]);
        const int axis = (ex >= ey && ex >= ez) ? 0 : (ey >= ez ? 1 : 2);
        const double ext = axis == 0 ? ex : (axis == 1 ? ey : ez);
        uint32_t l = 0;
        if (cn <= RT_LEAF_MAX || ext <= 1e-7 || !alloc_pair(A, static_cast<int>(t), l)) {
          S.axis[i] = -1;  // leaf (degenerate centroids, or no node capacity left)
          A.nsplit[id] = -1;
          unsigned long long k[6];
          rt_keys_empty(k);
          for (int j = 0; j < cn; ++j) rt_fold_box(A.tiles[t], S.idx[S.off[cur][i] + j], k);
          rt_store_box(A, id, k);
        } else {
          A.P[s + static_cast<uint32_t>(atomicAdd(&S.nint, 1))] = id;  // its box after the last level
          const double ca = axis == 0 ? clo[0] : (axis == 1 ? clo[1] : clo[2]);
          const double cb = axis == 0 ? chi[0] : (axis == 1 ? chi[1] : chi[2]);
          const double mid = __dmul_rn(0.5, __dadd_rn(ca, cb));
          S.axis[i] = static_cast<int8_t>(axis);
          S.mid[i] = mid;
          S.child[i] = static_cast<uint32_t>(nb + l);
          A.nsplit[id] = axis;
          A.nmid[id] = mid;
          A.nchild[id] = make_int2(static_cast<int>(nb + l), static_cast<int>(nb + l + 1));
          A.parent[nb + l] = id;
          A.parent[nb + l + 1] = id;
        }
      }
      __syncthreads();
      if (tid == 0) {
        if (S.nlvl < RT_CTA_LVMAX) S.lvend[S.nlvl++] = static_cast<uint16_t>(S.nint);
        else atomicOr(A.err, ERR_STACK_OVERFLOW);  // deeper than the depth check allows
      }
      // Flags and their exclusive prefix sum: thread tid owns positions RT_CTA_PER * tid + k.
      {
        uint32_t f[RT_CTA_PER], sum = 0;
#pragma unroll
        for (int k = 0; k < RT_CTA_PER; ++k) {
          const int x = RT_CTA_PER * tid + k;
          const uint32_t node = S.nd[x];
          f[k] = 0;
          if (node != RT_CTA_FREE && S.axis[node] >= 0)
            f[k] = S.key[S.axis[node]][S.home[x]] < ord64(S.mid[node]) ? 0u : 1u;
          sum += f[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        if (lane == 31) S.scan[w] = incl;
        __syncthreads();
        uint32_t acc = incl - sum;
        for (int i = 0; i < w; ++i) acc += S.scan[i];
#pragma unroll
        for (int k = 0; k < RT_CTA_PER; ++k) {
          const int x = RT_CTA_PER * tid + k;
          S.flag[x] = static_cast<uint8_t>(f[k]);
          S.u.r.bb[x] = static_cast<uint16_t>(acc);
          acc += f[k];
        }
        if (tid == RT_CTA_T - 1) S.u.r.bb[RT_CTA_MAX] = static_cast<uint16_t>(acc);
      }
      __syncthreads();
      // Ranks P / Q; the children of every splitting node go to the next level (more than four
      // elements) or become small leaves.
      for (int x = tid; x < RT_CTA_MAX; x += RT_CTA_T) {
        const uint32_t node = S.nd[x];
        if (node == RT_CTA_FREE || S.axis[node] < 0) continue;
        const int o0 = S.off[cur][node], cn = S.cnt[cur][node];
        const int r = x - o0;
        const int bs = S.u.r.bb[o0];
        const int Bb = S.u.r.bb[x] - bs, Bt = S.u.r.bb[o0 + cn] - bs, St = cn - Bt;
        if (S.flag[x]) {
          S.u.r.P[o0 + Bb] = static_cast<uint16_t>(r);
        } else {
          S.u.r.Q[o0 + (St - (r - Bb)) - 1] = static_cast<uint16_t>(r);
        }
      }
      for (int i = tid; i < nl; i += RT_CTA_T) {
        if (S.axis[i] < 0) continue;
        const int o0 = S.off[cur][i], cn = S.cnt[cur][i];
        const int St = cn - (S.u.r.bb[o0 + cn] - S.u.r.bb[o0]);
        const int Sp = (St == 0 || St == cn) ? cn / 2 : St;  // bvh.rs:260-265
        S.sp[i] = static_cast<uint16_t>(Sp);
        const uint32_t cd = min(static_cast<uint32_t>(S.dep[cur][i]) + 1u, 255u);  // saturates past the depth check
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const uint32_t cid = S.child[i] + static_cast<uint32_t>(c);
          const int coff = o0 + (c ? Sp : 0), csz = c ? cn - Sp : Sp;
          if (csz > RT_LEAF_MAX) {
            const int slot = atomicAdd(&S.nnext, 1);
            S.id[cur ^ 1][slot] = cid;
            S.off[cur ^ 1][slot] = static_cast<uint16_t>(coff);
            S.cnt[cur ^ 1][slot] = static_cast<uint16_t>(csz);
            S.dep[cur ^ 1][slot] = static_cast<uint8_t>(cd);
            S.cslot[i][c] = static_cast<uint8_t>(slot);
          } else {
            const int qi = atomicAdd(&S.nslnew, 1);
            S.sl[qi] = static_cast<uint32_t>(coff) | static_cast<uint32_t>(csz) << 11 | cd << 14;
            S.slid[qi] = cid;
            S.cslot[i][c] = RT_CTA_FREE;
          }
        }
      }
      __syncthreads();
      // Place: every element of a splitting node moves to its place after the swap partition.
      uint16_t vp[RT_CTA_PER];
      uint32_t vi[RT_CTA_PER];
      int dst[RT_CTA_PER];
      uint8_t vn[RT_CTA_PER];
#pragma unroll
      for (int k = 0; k < RT_CTA_PER; ++k) {
        const int x = k * RT_CTA_T + tid;
        const uint32_t node = S.nd[x];
        dst[k] = -1;
        vn[k] = RT_CTA_FREE;
        if (node == RT_CTA_FREE) continue;
        vp[k] = S.home[x];
        vi[k] = S.idx[x];
        if (S.axis[node] < 0) {  // a leaf of this level: its order is final
          dst[k] = x;
          continue;
        }
        const int o0 = S.off[cur][node], cn = S.cnt[cur][node];
        const int r = x - o0;
        const int bs = S.u.r.bb[o0];
        const int Bb = S.u.r.bb[x] - bs, Bt = S.u.r.bb[o0 + cn] - bs, St = cn - Bt;
        const int li = St + (St < cn ? S.flag[o0 + St] : 0);
        const bool big = S.flag[x] != 0;
        int d;
        if (r < li) {
          d = big ? ((Bb == 0 ? cn : S.u.r.Q[o0 + Bb - 1]) - 1) : r;
        } else {
          d = big ? r - 1 : S.u.r.P[o0 + (St - (r - Bb)) - 1];
        }
        dst[k] = o0 + d;
        vn[k] = S.cslot[node][d < S.sp[node] ? 0 : 1];
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < RT_CTA_PER; ++k) {
        if (dst[k] < 0) continue;
        S.home[dst[k]] = vp[k];
        S.idx[dst[k]] = vi[k];
        S.nd[dst[k]] = vn[k];
      }
      if (tid == 0) {
        S.nl = S.nnext;
        S.nsl = S.nslnew;
      }
      cur ^= 1;
      __syncthreads();
    }
    // The internal nodes' boxes, deepest level first: each the union of its children's, written
    // by this block before the barrier (leaves at their creation, internal nodes a level below).
    for (int L = S.nlvl - 1; L >= 0; --L) {
      const int b0 = L ? S.lvend[L - 1] : 0, b1 = S.lvend[L];
      for (int k = b0 + tid; k < b1; k += RT_CTA_T) {
        const uint32_t id = A.P[s + static_cast<uint32_t>(k)];
        const int2 ch = A.nchild[id];
        const double* a = A.box64 + 6ull * static_cast<unsigned long long>(ch.x);
        const double* b = A.box64 + 6ull * static_cast<unsigned long long>(ch.y);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          A.box64[6ull * id + m] = unord64(umin64(ord64(a[m]), ord64(b[m])));
          A.box64[6ull * id + 3 + m] = unord64(umax64(ord64(a[3 + m]), ord64(b[3 + m])));
        }
      }
      __syncthreads();
    }
    for (int x = tid; x < n; x += RT_CTA_T) A.ridx[s + x] = S.idx[x];
    if (tid == 0) atomicMax(&A.tiles[t].depth, S.maxdep);
    __syncthreads();
  }
}

// Node boxes above the blocks' subtrees (the BVHNode aabb: the union of the node's elements'
// max_dim boxes, bvh.rs:196-204).  Every block-queue entry (a subtree's root, or a leaf of the
// global levels) has its box; one thread per entry climbs: at each parent the first child to
// arrive stops and the second forms the parent's box as the union of both children's.  Boxes are
// published with a fence before the arrival count and read through L2.  `arrive` holds one zeroed
// counter per node.
__global__ void k_rt_refit(RtArgs A, uint32_t* arrive) {
  const uint32_t nq = A.cnt[2];
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    unsigned long long node = A.bq[q];
    if (node >= A.N) {
      atomicOr(A.err, ERR_BAD_INDEX);
      continue;
    }
    const RTile& T = A.tiles[A.ntile[node]];
    const unsigned long long nlo = T.nbase, nhi = T.nbase + T.ncap;
    for (int up = 0; up <= RT_MAX_DEPTH; ++up) {
      const uint32_t p = A.parent[node];
      if (p == RT_NONE) break;
      if (p < nlo || p >= nhi) {
        atomicOr(A.err, ERR_BAD_INDEX);
        break;
      }
      __threadfence();
      if (atomicAdd(&arrive[p], 1u) == 0u) break;  // the other child forms the parent's box
      __threadfence();
      const int2 ch = A.nchild[p];
      if (static_cast<unsigned long long>(ch.x) < nlo || static_cast<unsigned long long>(ch.y) >= nhi) {
        atomicOr(A.err, ERR_BAD_INDEX);
        break;
      }
      const double* a = A.box64 + 6ull * static_cast<unsigned long long>(ch.x);
      const double* b = A.box64 + 6ull * static_cast<unsigned long long>(ch.y);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const unsigned long long l = umin64(ord64(__ldcg(a + m)), ord64(__ldcg(b + m)));
        const unsigned long long h = umax64(ord64(__ldcg(a + 3 + m)), ord64(__ldcg(b + 3 + m)));
        A.box64[6ull * p + m] = unord64(l);
        A.box64[6ull * p + 3 + m] = unord64(h);
      }
      node = p;
    }
  }
}

// Walk records (fg_rtree.cuh): one thread per node.  A leaf fills its element range and the
// leaf-of map; the root and every internal node at odd depth write their four-wide record, the
// grandchildren in the reference's visiting order (right before left, a leaf child in one slot).
// An internal slot's box is rounded outward, padded and extended by the reach; a leaf slot's box
// is rounded to nearest.
__global__ void k_rt_records(RtArgs A, Node4* rec, uint2* rleaf, uint32_t* leafof, unsigned long long leafof_n) {
  const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
  for (unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; g < A.N;
       g += stride) {
    int lo_ = 0, hi_ = A.ntiles - 1;
    while (lo_ < hi_) {
      const int mid = (lo_ + hi_ + 1) >> 1;
      if (A.tiles[mid].nbase <= g) lo_ = mid; else hi_ = mid - 1;
    }
    const RTile& T = A.tiles[lo_];
    const uint32_t id = static_cast<uint32_t>(g - T.nbase);
    // (After a failed node allocation, ids below the capacity may never have been set up; the
    // build has flagged the error, and the checks below keep this pass inside its buffers.)
    if (id >= min(T.nodes, T.ncap)) continue;
    Node4* R = rec + T.rbase;
    float bx[6][4];
    int ref[4] = {INT32_MIN, INT32_MIN, INT32_MIN, INT32_MIN};
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int c = 0; c < 6; ++c) bx[c][k] = 0.0f;
    auto put = [&](int k, Node4* out) {
      Node4 nd;
      nd.lox = make_float4(bx[0][0], bx[0][1], bx[0][2], bx[0][3]);
      nd.loy = make_float4(bx[1][0], bx[1][1], bx[1][2], bx[1][3]);
      nd.loz = make_float4(bx[2][0], bx[2][1], bx[2][2], bx[2][3]);
      nd.hix = make_float4(bx[3][0], bx[3][1], bx[3][2], bx[3][3]);
      nd.hiy = make_float4(bx[4][0], bx[4][1], bx[4][2], bx[4][3]);
      nd.hiz = make_float4(bx[5][0], bx[5][1], bx[5][2], bx[5][3]);
      nd.ref = make_int4(ref[0], ref[1], ref[2], ref[3]);
      nd._pad = make_int4(k, 0, 0, 0);
      *out = nd;
    };
    if (id == 0) {  // the super-root slot: an empty tree's record 0
      if (T.n == 0 && T.rcap > 0) put(0, R);
      continue;
    }
    if (id == 1 && T.n == 0) continue;
    const bool leaf = A.nsplit[g] < 0;
    if (leaf) {
      const uint32_t st = A.nstart[g], cn = A.ncount[g];
      if (st < T.ebase || st - T.ebase + static_cast<unsigned long long>(cn) > T.n) {
        atomicOr(A.err, ERR_BAD_INDEX);
        continue;
      }
      rleaf[g] = make_uint2(static_cast<uint32_t>(st - T.ebase), cn);
      if (leafof)
        for (uint32_t k = 0; k < cn; ++k) {
          const uint32_t slot = A.ridx[st + k];
          if (T.ebase + slot < leafof_n) leafof[T.ebase + slot] = id; else atomicOr(A.err, ERR_BAD_INDEX);
        }
    }
    if (id != 1 && (leaf || !(A.ndepth[g] & 1u))) continue;
    // Slot k takes node c (a global id inside the tile): its box and reference.
    int k = 0;
    bool bad = false;
    auto add = [&](unsigned long long c) {
      if (c < T.nbase || c >= T.nbase + T.ncap || k >= 4) {
        bad = true;
        return;
      }
      const double* b = A.box64 + 6ull * c;
      const int local = static_cast<int>(c - T.nbase);
      float f[6];
      if (A.nsplit[c] < 0) {
#pragma unroll
        for (int m = 0; m < 6; ++m) f[m] = __double2float_rn(b[m]);
        ref[k] = ~local;
      } else {
        const int2 ch = A.nchild[c];
        const long long r = (static_cast<long long>(ch.x) - static_cast<long long>(T.nbase)) >> 1;
        if (r < 1 || r >= static_cast<long long>(T.rcap)) {
          bad = true;
          return;
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          f[m] = __double2float_rd(b[m]) - T.pad - T.reach;
          f[3 + m] = __double2float_ru(b[3 + m]) + T.pad + T.reach;
        }
        ref[k] = static_cast<int>(r);
      }
#pragma unroll
      for (int m = 0; m < 6; ++m) bx[m][k] = f[m];
      ++k;
    };
    unsigned long long at = 0;  // record index
    if (leaf) {  // a root leaf
      add(g);
    } else {
      const int2 ch = A.nchild[g];
      if (id != 1) at = (static_cast<unsigned long long>(ch.x) - T.nbase) >> 1;
      const unsigned long long cs[2] = {static_cast<unsigned long long>(ch.y), static_cast<unsigned long long>(ch.x)};
#pragma unroll
      for (int q = 0; q < 2; ++q) {  // right child first
        const unsigned long long c = cs[q];
        if (c < T.nbase || c >= T.nbase + T.ncap) {
          bad = true;
          break;
        }
        if (A.nsplit[c] < 0) {
          add(c);
        } else {
          const int2 gc = A.nchild[c];
          add(static_cast<unsigned long long>(gc.y));
          add(static_cast<unsigned long long>(gc.x));
        }
      }
    }
    if (bad || at >= T.rcap) {
      atomicOr(A.err, ERR_BAD_INDEX);
      continue;
    }
    put(k, R + at);
  }
}

__global__ void k_rt_depth_check(RtArgs A) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < A.ntiles && A.tiles[t].depth > static_cast<uint32_t>(RT_MAX_DEPTH)) atomicOr(A.err, ERR_STACK_OVERFLOW);
}

}  // namespace

RtArgs rt_args(RTreeBufs& B, uint32_t* err) {
  RtArgs A;
  A.tiles = B.tiles.p;
  A.ntiles = B.ntiles;
  A.E = B.E;
  A.N = B.N;
  A.idx[0] = B.idx0.p;
  A.idx[1] = B.idx1.p;
  A.key[0] = B.key0.p;
  A.key[1] = B.key1.p;
  A.nof[0] = B.nof0.p;
  A.nof[1] = B.nof1.p;
  A.flag = B.flag.p;
  A.bb = B.bb.p;
  A.blk = B.blk.p;
  A.P = B.P.p;
  A.Q = B.Q.p;
  A.ridx = B.ridx.p;
  A.acc = B.acc.p;
  A.box64 = B.box64.p;
  A.parent = B.parent.p;
  A.nstart = B.nstart.p;
  A.ncount = B.ncount.p;
  A.ntile = B.ntile.p;
  A.ndepth = B.ndepth.p;
  A.nsplit = B.nsplit.p;
  A.nmid = B.nmid.p;
  A.nchild = B.nchild.p;
  A.wl[0] = B.wl0.p;
  A.wl[1] = B.wl1.p;
  A.bq = B.bq.p;
  A.bqpar = B.bqpar.p;
  A.cnt = B.cnt.p;
  A.err = err;
  return A;
}

void rtree_alloc(RTreeBufs& B, std::vector<RTile>& tiles, bool want_leafof, cudaStream_t st, double node_frac,
                 size_t leafof_slots) {
  B.ntiles = static_cast<int>(tiles.size());
  unsigned long long e = 0, nn = 0;
  uint32_t emax = 0;
  unsigned long long rr = 0;
  for (auto& t : tiles) {
    t.ebase = e;
    t.ncap = static_cast<uint32_t>(std::min<double>(t.ecap + 2.0, std::ceil(t.ecap * node_frac) + 64.0));
    t.nbase = nn;
    t.rcap = t.ncap / 2 + 1;
    t.rbase = static_cast<uint32_t>(rr);
    e += t.ecap;
    nn += t.ncap;
    rr += t.rcap;
    emax = std::max(emax, t.ecap);
  }
  FG_REQUIRE(e < 0x7fffffffull && nn < 0x7fffffffull, "too many elements for one reference-tree build");
  B.E = e;
  B.N = nn;
  B.R = rr;
  B.levels = levels_for(emax);
  const size_t E1 = static_cast<size_t>(std::max<unsigned long long>(e, 1));
  const size_t N1 = static_cast<size_t>(std::max<unsigned long long>(nn, 1));
  B.tiles.alloc(tiles.size(), st);
  FG_CUDA(cudaMemcpyAsync(B.tiles.p, tiles.data(), tiles.size() * sizeof(RTile), cudaMemcpyHostToDevice, st));
  B.idx0.alloc(E1, st);
  B.idx1.alloc(E1, st);
  B.key0.alloc(3 * E1, st);
  B.key1.alloc(3 * E1, st);
  B.nof0.alloc(E1, st);
  B.nof1.alloc(E1, st);
  B.flag.alloc(E1 + 1, st);
  B.bb.alloc(E1 + 1, st);
  B.nblk = (E1 + 1 + SCAN_ITEMS - 1) / SCAN_ITEMS;
  B.blk.alloc(B.nblk, st);
  B.P.alloc(E1, st);
  B.Q.alloc(E1, st);
  B.ridx.alloc(E1, st);
  B.acc.alloc(6 * N1, st);
  B.box64.alloc(6 * N1, st);
  B.parent.alloc(N1, st);
  B.nstart.alloc(N1, st);
  B.ncount.alloc(N1, st);
  B.ntile.alloc(N1, st);
  B.ndepth.alloc(N1, st);
  B.nsplit.alloc(N1, st);
  B.nmid.alloc(N1, st);
  B.nchild.alloc(N1, st);
  B.wl0.alloc(N1, st);
  B.wl1.alloc(N1, st);
  B.bq.alloc(N1, st);
  B.bqpar.alloc(N1, st);
  B.cnt.alloc(4, st);
  B.rnode.alloc(std::max<unsigned long long>(rr, 1), st);
  B.rleaf.alloc(N1, st);
  if (want_leafof) B.leafof.alloc(std::max(E1, leafof_slots), st);
  FG_CUDA(cudaMemsetAsync(B.ridx.p, 0, E1 * sizeof(uint32_t), st));
}

namespace {

// Carves the buffers of a one-tile tree from `base` (or only counts the bytes when base is null).
size_t carve(RTreeBufs* B, uint32_t ecap, bool want_leafof, uint32_t leafof_slots, unsigned char* base) {
  const size_t E1 = std::max<uint32_t>(ecap, 1);
  const size_t N1 = rt_attach_nodes(E1);
  const size_t nblk = rt_attach_blocks(E1);
  static_assert(SCAN_ITEMS == 2048, "rt_attach_blocks assumes 2048 entries per prefix-sum block");
  size_t off = 0;
  auto take = [&](auto& buf, size_t count) {
    using T = typename std::remove_reference<decltype(*buf.p)>::type;
    off = (off + 255) / 256 * 256;
    if (base) buf.view(reinterpret_cast<T*>(base + off), count);
    off += count * sizeof(T);
  };
  RTreeBufs dummy;
  RTreeBufs& b = B ? *B : dummy;
  take(b.tiles, 1);
  take(b.idx0, E1);
  take(b.idx1, E1);
  take(b.key0, 3 * E1);
  take(b.key1, 3 * E1);
  take(b.nof0, E1);
  take(b.nof1, E1);
  take(b.flag, E1 + 1);
  take(b.bb, E1 + 1);
  take(b.blk, nblk);
  take(b.P, E1);
  take(b.Q, E1);
  take(b.ridx, E1);
  take(b.acc, 6 * N1);
  take(b.box64, 6 * N1);
  take(b.parent, N1);
  take(b.nstart, N1);
  take(b.ncount, N1);
  take(b.ntile, N1);
  take(b.ndepth, N1);
  take(b.nsplit, N1);
  take(b.nmid, N1);
  take(b.nchild, N1);
  take(b.wl0, N1);
  take(b.wl1, N1);
  take(b.bq, N1);
  take(b.bqpar, N1);
  take(b.cnt, 4);
  take(b.rnode, N1 / 2 + 1);
  take(b.rleaf, N1);
  if (want_leafof) take(b.leafof, std::max<uint32_t>(leafof_slots, 1));
  if (B) {
    B->ntiles = 1;
    B->E = E1;
    B->N = N1;
    B->R = N1 / 2 + 1;
    B->nblk = nblk;
    B->levels = levels_for(ecap);
  }
  return (off + 255) / 256 * 256;
}

}  // namespace

size_t rtree_scratch_bytes(uint32_t ecap, bool want_leafof, uint32_t leafof_slots) {
  return carve(nullptr, ecap, want_leafof, leafof_slots, nullptr);
}

void rtree_attach(RTreeBufs& B, RTile tile, bool want_leafof, uint32_t leafof_slots, unsigned char* base,
                  size_t bytes, cudaStream_t st) {
  const size_t need = carve(nullptr, tile.ecap, want_leafof, leafof_slots, nullptr);
  FG_REQUIRE(need == rtree_attach_bytes(tile.ecap, want_leafof, leafof_slots), "tree scratch layout mismatch");
  FG_REQUIRE(need <= bytes, "tree scratch too small");
  carve(&B, tile.ecap, want_leafof, leafof_slots, base);
  tile.ebase = 0;
  tile.nbase = 0;
  tile.ncap = static_cast<uint32_t>(B.N);
  tile.rbase = 0;
  tile.rcap = static_cast<uint32_t>(B.R);
  FG_CUDA(cudaMemcpyAsync(B.tiles.p, &tile, sizeof(RTile), cudaMemcpyHostToDevice, st));
}

void rtree_build(RTreeBufs& B, uint32_t* err, cudaStream_t st, RTile* tiles_dev) {
  if (B.ntiles == 0) return;
  RtArgs A = rt_args(B, err);
  if (tiles_dev) A.tiles = tiles_dev;
  const unsigned G = static_cast<unsigned>(std::min<unsigned long long>((B.E + RT_BLOCK) / RT_BLOCK, 152ull * 16));
  const unsigned GN = static_cast<unsigned>(std::min<unsigned long long>((B.N + RT_BLOCK - 1) / RT_BLOCK, 152ull * 16));
  const unsigned GS = static_cast<unsigned>(std::min<unsigned long long>(B.nblk, 152ull * 16));
  FG_CUDA(cudaMemsetAsync(B.cnt.p, 0, 4 * sizeof(uint32_t), st));
  k_rt_init<<<G, RT_BLOCK, 0, st>>>(A);
  for (int L = 0; L < B.levels; ++L) {
    const int c = L & 1;
    k_rt_reduce<<<G, RT_BLOCK, 0, st>>>(A, c);
    k_rt_decide<<<GN, RT_BLOCK, 0, st>>>(A, c);
    k_rt_scan_blocks<<<GS, RT_BLOCK, 0, st>>>(A, c, B.nblk);
    k_rt_scan_top<<<1, 1024, 0, st>>>(A, c, B.nblk);
    k_rt_scan_final<<<GS, RT_BLOCK, 0, st>>>(A, c, B.nblk);
    k_rt_pq<<<G, RT_BLOCK, 0, st>>>(A, c);
    k_rt_place<<<G, RT_BLOCK, 0, st>>>(A, c);
    k_rt_level_end<<<1, 1, 0, st>>>(A, c);
  }
  k_rt_check<<<1, 1, 0, st>>>(A, B.levels & 1);
  const unsigned GC = static_cast<unsigned>(
      std::min<unsigned long long>(B.E / (RT_LEAF_MAX + 1) + static_cast<unsigned long long>(B.ntiles), 152ull * 8));
  static_assert(sizeof(RtCtaSmem) <= 56 * 1024, "four blocks of the block phase must fit an SM");
  FG_CUDA(cudaFuncSetAttribute(k_rt_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(sizeof(RtCtaSmem))));
  k_rt_cta<<<GC, RT_CTA_T, sizeof(RtCtaSmem), st>>>(A);
  // The global worklist is spent: its words count the children that reached each node.
  FG_CUDA(cudaMemsetAsync(B.wl0.p, 0, static_cast<size_t>(B.N) * sizeof(uint32_t), st));
  k_rt_refit<<<GN, RT_BLOCK, 0, st>>>(A, B.wl0.p);
  k_rt_records<<<GN, RT_BLOCK, 0, st>>>(A, B.rnode.p, B.rleaf.p, B.leafof.p, B.leafof.n);
  k_rt_depth_check<<<grid_for(static_cast<size_t>(B.ntiles), 128), 128, 0, st>>>(A);
  FG_CUDA(cudaGetLastError());
}

// Element lists of an emulsion in crystal-id order: all crystals (their slots), or the developed
// ones (flag, exclusive sum, scatter).
__global__ void k_rt_id_slots(const uint32_t* id2s, uint32_t n, const uint8_t* developed, uint32_t* flag) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = id2s ? id2s[k] : k;
  flag[k] = developed[s] ? 1u : 0u;
}
__global__ void k_rt_id_scatter(const uint32_t* id2s, uint32_t n, const uint32_t* flag, const uint32_t* pos,
                                uint32_t* list) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !flag[k]) return;
  list[pos[k]] = id2s ? id2s[k] : k;
}

void build_emulsion_tree(fg_engine* e, const fg_emulsion* em, bool developed_only, RTreeBufs& B,
                         DBuf<uint32_t>& list) {
  cudaStream_t st = e->stream;
  const uint32_t n = em->n;
  RTile t{};
  t.a = em->a.p;
  t.d = em->d.p;
  t.pos64 = em->has64 ? em->pos64.p : nullptr;
  t.dims64 = em->has64 ? em->dims64.p : nullptr;
  t.exp64 = developed_only ? em->exp64.p : nullptr;
  t.pad = static_cast<float>(std::max(em->extent, std::max(em->cfg.width, em->cfg.height)) * 2e-6 + 1e-5);
  t.reach = developed_only ? 0.0f : rt_reach(em->any_cubic ? em->max_half_dim : 0.0);
  const uint32_t* id2s = em->h_s2id.empty() ? nullptr : em->id_to_sorted.p;
  uint32_t m = n;
  if (developed_only && n) {
    DBuf<uint32_t> flag(n + 1, st), pos(n + 1, st);
    FG_CUDA(cudaMemsetAsync(flag.p + n, 0, sizeof(uint32_t), st));
    k_rt_id_slots<<<grid_for(n, 256), 256, 0, st>>>(id2s, n, em->developed.p, flag.p);
    exclusive_scan_u32(flag.p, pos.p, n + 1, st);
    FG_CUDA(cudaMemcpyAsync(&m, pos.p + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    list.alloc(std::max<uint32_t>(m, 1), st);
    k_rt_id_scatter<<<grid_for(n, 256), 256, 0, st>>>(id2s, n, flag.p, pos.p, list.p);
    FG_CUDA(cudaGetLastError());
    t.order = list.p;
  } else {
    t.order = id2s;
  }
  t.ecap = developed_only ? std::max<uint32_t>(m, 1) : std::max<uint32_t>(n, 1);
  t.n = developed_only ? m : n;
  std::vector<RTile> v{t};
  rtree_alloc(B, v, developed_only, st, 1.0, n);
  rtree_build(B, e->d_err, st);
  B.count = t.n;
}

unsigned rtree_kernel_launches(const RTreeBufs& B) {
  return B.ntiles ? 1u + 8u * static_cast<unsigned>(B.levels) + 5u : 0u;
}

}  // namespace fg

extern "C" fg_status fg_emulsion_reference_tree(fg_engine* e, const fg_emulsion* em, int developed_only,
                                                uint32_t* order, uint32_t* leaves, double* leaf_boxes, size_t cap,
                                                size_t* nelem, size_t* nleaves) {
  using namespace fg;
  return guard(e, [&] {
    FG_REQUIRE(em, "null emulsion");
    cudaStream_t st = e->stream;
    begin_call(e);
    RTreeBufs local;
    DBuf<uint32_t> list;
    const RTreeBufs* T = &em->rt;
    if (developed_only) {
      build_emulsion_tree(e, em, true, local, list);
      T = &local;
    }
    RTile tile{};
    if (T->ntiles) FG_CUDA(cudaMemcpyAsync(&tile, T->tiles.p, sizeof(RTile), cudaMemcpyDeviceToHost, st));
    FG_CUDA(cudaStreamSynchronize(st));
    end_call(e);  // raises a build error first
    const uint32_t n = T->ntiles ? tile.n : 0, nn = T->ntiles ? std::min(tile.nodes, tile.ncap) : 0;
    std::vector<uint32_t> ridx(n), nstart(nn), ncount(nn);
    std::vector<int> nsplit(nn);
    std::vector<double> box(6ull * nn);
    if (n) FG_CUDA(cudaMemcpyAsync(ridx.data(), T->ridx.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (nn) {
      FG_CUDA(cudaMemcpyAsync(nstart.data(), T->nstart.p, nn * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(ncount.data(), T->ncount.p, nn * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(nsplit.data(), T->nsplit.p, nn * sizeof(int), cudaMemcpyDeviceToHost, st));
      FG_CUDA(cudaMemcpyAsync(box.data(), T->box64.p, 6ull * nn * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    FG_CUDA(cudaStreamSynchronize(st));
    if (nelem) *nelem = n;
    if (order)
      for (uint32_t k = 0; k < n && k < cap; ++k) order[k] = em->h_s2id.empty() ? ridx[k] : em->h_s2id[ridx[k]];
    std::vector<uint32_t> lf;
    for (uint32_t id = 1; id < nn && n; ++id)
      if (nsplit[id] < 0) lf.push_back(id);
    std::sort(lf.begin(), lf.end(), [&](uint32_t a, uint32_t b) { return nstart[a] < nstart[b]; });
    if (nleaves) *nleaves = lf.size();
    for (size_t k = 0; k < lf.size() && k < cap; ++k) {
      if (leaves) {
        leaves[2 * k] = nstart[lf[k]];
        leaves[2 * k + 1] = ncount[lf[k]];
      }
      if (leaf_boxes)
        for (int j = 0; j < 6; ++j) leaf_boxes[6 * k + j] = box[6ull * lf[k] + j];
    }
  });
}
