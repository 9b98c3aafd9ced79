// Device crystal synthesis: column-parallel Bridson, thinning to the reference density, Morton
// compaction and crystal attributes.  See fg_synth.cuh for the scheme.
#include <algorithm>

#include "fg_internal.h"
#include "fg_synth.cuh"

namespace fg {

enum : uint32_t {
  TAG_CAND = 0x43410000u,
  TAG_SEED = 0x53450000u,
  TAG_THIN = 0x54480000u,
};

// True when the cell word w holds a point closer than r to the candidate at (lx, ly, lz) (fixed
// point, relative to the candidate's cell) from the cell at offset (dx, dy, dz).
__device__ __forceinline__ bool syn_conflict(uint32_t w, int dx, int dy, int dz, int lx, int ly, int lz) {
  if (!(w & OCC)) return false;
  const int ex = dx * SYN_Q + static_cast<int>(w & 1023u) - lx;
  const int ey = dy * SYN_Q + static_cast<int>((w >> 10) & 1023u) - ly;
  const int ez = dz * SYN_Q + static_cast<int>((w >> 20) & 1023u) - lz;
  return ex * ex + ey * ey + ez * ez < SYN_R2X;
}

// First half of the candidate test, one lane per candidate: the 27 cells of the inner 3x3x3 block
// (the candidate's own cell first).  They reject about 87 % of Bridson candidates, so the lanes
// that survive are few and the rest of the test runs warp-cooperatively (syn_outer_free).
__device__ __forceinline__ bool syn_near_free(const uint32_t* grid, int rb, int lx, int ly, int lz) {
  if (syn_conflict(grid[rb], 0, 0, 0, lx, ly, lz)) return false;
#pragma unroll
  for (int k = 0; k < 27; ++k) {
    if (k == 13) continue;
    const int dx = k % 3 - 1, dy = (k / 3) % 3 - 1, dz = k / 9 - 1;
    if (syn_conflict(grid[rb + (dz * SYN_R + dy) * SYN_R + dx], dx, dy, dz, lx, ly, lz)) return false;
  }
  return true;
}

// The 90 cells of the 5x5x5 neighbourhood outside the inner block (without its eight corners,
// which cannot hold a point within r = sqrt(3) cells), as packed entries: region-index offset in
// the low 16 bits (signed), dx + 2, dy + 2, dz + 2 in three bits each from bit 16.
constexpr int SYN_OUTER = 90;

__device__ void syn_outer_table(int* tbl) {
  int j = 0;
  for (int dz = -2; dz <= 2; ++dz)
    for (int dy = -2; dy <= 2; ++dy)
      for (int dx = -2; dx <= 2; ++dx) {
        const int ax = dx < 0 ? -dx : dx, ay = dy < 0 ? -dy : dy, az = dz < 0 ? -dz : dz;
        if (ax < 2 && ay < 2 && az < 2) continue;
        if (ax == 2 && ay == 2 && az == 2) continue;
        tbl[j++] = (((dz * SYN_R + dy) * SYN_R + dx) & 0xffff) | ((dx + 2) << 16) | ((dy + 2) << 19) | ((dz + 2) << 22);
      }
}

// Whether the candidate at region cell cb, fixed-point offsets (cx, cy, cz) inside it, has a point
// within r in the 90 outer cells; the warp splits the cells over its lanes.  All 32 lanes call it
// with the same candidate; the answer is the same in every lane.
__device__ __forceinline__ bool syn_outer_hit(const uint32_t* grid, const int* tbl, int cb, int cx, int cy, int cz,
                                              int lane) {
  bool hit = false;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int j = lane + 32 * k;
    if (j < SYN_OUTER) {
      const int e = tbl[j];
      hit |= syn_conflict(grid[cb + static_cast<int16_t>(e & 0xffff)], ((e >> 16) & 7) - 2, ((e >> 19) & 7) - 2,
                          ((e >> 22) & 7) - 2, cx, cy, cz);
    }
  }
  return __any_sync(0xffffffffu, hit);
}

// Second half of the test for the lanes whose candidates passed syn_near_free: the warp takes the
// survivors one at a time, in lane order, until one also passes the outer cells: the step's first
// valid candidate, the only lane left valid.  The survivors after it stay untested (`rest`, the
// same in every lane): the round's resolution needs another candidate only when that one
// conflicts with a point accepted for an earlier warp, and tests them then.  All 32 lanes call it.
__device__ __forceinline__ bool syn_outer_free(const uint32_t* grid, const int* tbl, bool valid, int rb, int lx,
                                               int ly, int lz, int lane, unsigned& rest) {
  unsigned sm = __ballot_sync(0xffffffffu, valid);
  int win = -1;
  while (sm) {
    const int c = __ffs(sm) - 1;
    sm &= sm - 1;
    const int cb = __shfl_sync(0xffffffffu, rb, c);
    const int cx = __shfl_sync(0xffffffffu, lx, c);
    const int cy = __shfl_sync(0xffffffffu, ly, c);
    const int cz = __shfl_sync(0xffffffffu, lz, c);
    if (!syn_outer_hit(grid, tbl, cb, cx, cy, cz, lane)) {
      win = c;
      break;
    }
  }
  rest = sm;
  return lane == win;
}

// Exact test of a fixed-point candidate against the staged grid: every point within r.  The eight
// corner cells of the 5x5x5 neighbourhood cannot hold a point within r = sqrt(3) cells.  The
// outer loop stays rolled (small code), the first point within r ends the test.
__device__ __forceinline__ bool syn_free(const uint32_t* grid, int nz, int rx, int ry, int rz, int X, int Y, int Z,
                                         int cx, int cy, int cz, uint32_t* err) {
  // The neighbourhood must lie inside the staged region (it does for candidates within 2r of a
  // point of the column); a candidate that fails the check is rejected.
  if (!index_ok(rx >= 2 && rx <= SYN_R - 3 && ry >= 2 && ry <= SYN_R - 3 && rz >= 2 && rz <= nz - 3, err,
                SITE_SYN_REGION, static_cast<uint32_t>(rx | (ry << 8) | (rz << 16)), blockIdx.x))
    return false;
#pragma unroll 1
  for (int dz = -2; dz <= 2; ++dz) {
    const bool zedge = dz == -2 || dz == 2;
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
      const int row = ((rz + dz) * SYN_R + (ry + dy)) * SYN_R + rx;
#pragma unroll
      for (int dx = -2; dx <= 2; ++dx) {
        if (zedge && (dx == -2 || dx == 2) && (dy == -2 || dy == 2)) continue;
        const uint32_t w = grid[row + dx];
        if (w & OCC) {
          const int ex = (cx + dx) * SYN_Q + static_cast<int>(w & 1023u) - X;
          const int ey = (cy + dy) * SYN_Q + static_cast<int>((w >> 10) & 1023u) - Y;
          const int ez = (cz + dz) * SYN_Q + static_cast<int>((w >> 20) & 1023u) - Z;
          if (ex * ex + ey * ey + ez * ez < SYN_R2X) return false;
        }
      }
    }
  }
  return true;
}

__device__ __forceinline__ uint32_t syn_word(int X, int Y, int Z) {
  return OCC | (static_cast<uint32_t>(Z & 1023) << 20) | (static_cast<uint32_t>(Y & 1023) << 10) |
         static_cast<uint32_t>(X & 1023);
}

// Launch bounds of 8 CTAs per SM (32 registers): more columns in flight hide the round's barriers.
// A column with its one-cell spill and the halo stages 14 x 14 cells per layer, so eight CTAs fit
// in the SM's 228 KB of shared memory for depths up to 23 cells.
// All columns of all four colour classes in one launch, class after class in block order.  A column
// starts once the columns of lower classes next to it have written their cells back (their done
// flags), which gives every column the cell state it would see if the classes ran one launch
// after another: only the eight neighbouring columns share cells with it, and a neighbour of a
// higher class waits for it in turn.  The flags are waited on by lower block indices only, so
// the wait ends as the earlier blocks finish; it is bounded all the same (ERR_SPIN_LIMIT).
__global__ void __launch_bounds__(SYN_WARPS * 32, 8) k_bridson(const SynthTile* __restrict__ tiles,
                                                            int ntiles, uint4 class_base, int nz,
                                                            uint32_t* __restrict__ cells,
                                                            uint32_t* __restrict__ npts, uint32_t* done,
                                                            uint32_t* err, uint32_t wait_limit,
                                                            const uint32_t* probe) {
  extern __shared__ uint32_t syn_sm[];
  uint32_t* grid = syn_sm;                                   // SYN_R^2 * nz cell words
  uint16_t* active = reinterpret_cast<uint16_t*>(grid + SYN_R * SYN_R * nz);  // SYN_B^2 * (nz - 4)
  __shared__ int s_nact, s_wsum[SYN_WARPS];
  __shared__ int s_ncom;  // points this column commits (each fills one empty cell of its tile)
  __shared__ int s_pick[SYN_WARPS];
  __shared__ unsigned s_vmask[SYN_WARPS];  // the step's first valid candidate (at most one lane)
  __shared__ unsigned s_rmask[SYN_WARPS];  // later candidates that passed the near cells, untested
  __shared__ int s_cx[SYN_WARPS][32], s_cy[SYN_WARPS][32], s_cz[SYN_WARPS][32];  // valid candidates
  __shared__ int s_outer[SYN_OUTER];

  // Column of this CTA: colour class, tile, then the j-th column of this class in that tile.
  const uint32_t cb[4] = {class_base.x, class_base.y, class_base.z, class_base.w};
  const int color = blockIdx.x >= cb[3] ? 3 : (blockIdx.x >= cb[2] ? 2 : (blockIdx.x >= cb[1] ? 1 : 0));
  const uint32_t bidx = blockIdx.x - cb[color];
  int lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tiles[mid].col_base[color] <= bidx) lo = mid; else hi = mid - 1;
  }
  const SynthTile& t = tiles[lo];
  const uint32_t j = bidx - t.col_base[color];
  const uint32_t cxn = (t.nbx - (color & 1) + 1) / 2;
  const uint32_t bx = 2 * (j % cxn) + (color & 1), by = 2 * (j / cxn) + (color >> 1);
  const int x0 = static_cast<int>(bx) * SYN_B, y0 = static_cast<int>(by) * SYN_B;
  const int x1 = min(x0 + SYN_B, static_cast<int>(t.gw)), y1 = min(y0 + SYN_B, static_cast<int>(t.gh));
  const int gd = static_cast<int>(t.gd);
  const int ox = x0 - SYN_HALO, oy = y0 - SYN_HALO;
  const uint32_t colkey = by * t.nbx + bx;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ncell = SYN_R * SYN_R * nz;
  const int acap = SYN_B * SYN_B * (nz - 4);  // active list capacity: one entry per column cell
  uint32_t* tc = cells + t.cell_base;

  // Wait for the neighbouring columns of lower classes.
  if (tid == 0 && color > 0) {
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int nx = static_cast<int>(bx) + dx, ny = static_cast<int>(by) + dy;
        if ((dx == 0 && dy == 0) || nx < 0 || ny < 0 || nx >= static_cast<int>(t.nbx) || ny >= static_cast<int>(t.nby))
          continue;
        const int nc = (nx & 1) | ((ny & 1) << 1);
        if (nc >= color) continue;
        const uint32_t ncxn = (t.nbx - (nc & 1) + 1) / 2;
        const uint32_t id = cb[nc] + t.col_base[nc] + static_cast<uint32_t>(ny >> 1) * ncxn + static_cast<uint32_t>(nx >> 1);
        const volatile uint32_t* f = done + id;
        uint32_t spins = 0;
        while (*f == 0u) {
          if (++spins > wait_limit) {
            atomicOr(err, ERR_SPIN_LIMIT);
            break;
          }
          __nanosleep(64);
        }
      }
    __threadfence();
  }
  // Failure drill: a flag that nothing sets, waited on with the same bound.
  if (tid == 0 && probe) {
    const volatile uint32_t* f = probe;
    uint32_t spins = 0;
    while (*f == 0u) {
      if (++spins > wait_limit) {
        atomicOr(err, ERR_SPIN_LIMIT);
        break;
      }
      __nanosleep(64);
    }
  }
  __syncthreads();

  // Stage the region (column + halo) of the cell grid (through L2: neighbours wrote it).
  for (int i = tid; i < ncell; i += blockDim.x) {
    const int rx = i % SYN_R, ry = (i / SYN_R) % SYN_R, rz = i / (SYN_R * SYN_R);
    const int gx = ox + rx, gy = oy + ry, gz = rz - 2;
    uint32_t w = 0;
    if (gx >= 0 && gy >= 0 && gz >= 0 && gx < static_cast<int>(t.gw) && gy < static_cast<int>(t.gh) && gz < gd)
      w = __ldcg(tc + (static_cast<size_t>(gz) * t.gh + gy) * t.gw + gx);
    grid[i] = w;
  }
  if (tid == 0) {
    s_nact = 0;
    s_ncom = 0;
    syn_outer_table(s_outer);
  }
  __syncthreads();
  // Active list: the column's points in cell order (deterministic block-wide compaction).
  const int bw = x1 - x0, bh = y1 - y0;
  const int bcells = bw * bh * gd;
  for (int base = 0; base < bcells; base += blockDim.x) {
    const int i = base + tid;
    int ridx = 0;
    bool o = false;
    if (i < bcells) {
      const int lx = i % bw, ly = (i / bw) % bh, lz = i / (bw * bh);
      ridx = ((lz + 2) * SYN_R + (ly + SYN_HALO)) * SYN_R + (lx + SYN_HALO);
      o = (grid[ridx] & OCC) != 0;
    }
    const unsigned m = __ballot_sync(0xffffffffu, o);
    if (lane == 0) s_wsum[warp] = __popc(m);
    __syncthreads();
    int off = s_nact;
    for (int w = 0; w < warp; ++w) off += s_wsum[w];
    if (o) active[off + __popc(m & ((1u << lane) - 1u))] = static_cast<uint16_t>(ridx);
    __syncthreads();
    if (tid == 0)
      for (int w = 0; w < SYN_WARPS; ++w) s_nact += s_wsum[w];
    __syncthreads();
  }
  // An empty column starts from one random point (poisson.rs:46-57), up to 30 tries.
  if (tid == 0 && s_nact == 0 && bw > 0 && bh > 0) {
    for (int k = 0; k < SYN_K; ++k) {
      const P4 r = philox(static_cast<uint32_t>(k), 0, colkey, TAG_SEED, t.k0, t.k1);
      const int X = x0 * SYN_Q + static_cast<int>(uf(r.x) * static_cast<float>(bw * SYN_Q));
      const int Y = y0 * SYN_Q + static_cast<int>(uf(r.y) * static_cast<float>(bh * SYN_Q));
      const int Z = static_cast<int>(uf(r.z) * static_cast<float>(t.ZW));
      if (X >= static_cast<int>(t.XW) || Y >= static_cast<int>(t.YW) || Z >= static_cast<int>(t.ZW)) continue;
      const int cx = X >> 10, cy = Y >> 10, cz = Z >> 10;
      const int rx = cx - ox, ry = cy - oy, rz = cz + 2;
      if (!syn_free(grid, nz, rx, ry, rz, X, Y, Z, cx, cy, cz, err)) continue;
      const int ridx = (rz * SYN_R + ry) * SYN_R + rx;
      grid[ridx] = syn_word(X, Y, Z);
      ++s_ncom;
      if (index_ok(s_nact < acap, err, SITE_SYN_ACTIVE, s_nact, blockIdx.x)) active[s_nact++] = static_cast<uint16_t>(ridx);
      break;
    }
  }
  const int max_iter = 16 * SYN_B * SYN_B * gd + 64;
  for (int iter = 0;; ++iter) {
    __syncthreads();
    const int nact = s_nact;
    if (nact == 0) break;
    if (iter >= max_iter) {
      if (tid == 0) atomicOr(err, ERR_SPIN_LIMIT);
      break;
    }
    // One Bridson step per warp on a random active point (poisson.rs:59-129): 30 candidates in
    // the shell [r, 2r], one per lane; the lowest valid lane is the step's winner.  Every lane
    // draws one Philox block of the warp's stream: lanes 0-29 place the candidates and lane 31's
    // draw picks the active point (shuffled to the warp); lane 0 records the pick for the
    // retirement.
    static_assert(SYN_K < 32, "lane 31 draws the pick");
    const P4 r = philox(static_cast<uint32_t>(iter), static_cast<uint32_t>(warp * 32 + lane), colkey, TAG_CAND,
                        t.k0, t.k1);
    const uint32_t rpick = __shfl_sync(0xffffffffu, r.x, 31);
    const int pick = static_cast<int>((static_cast<unsigned long long>(rpick) * static_cast<unsigned>(nact)) >> 32);
    if (lane == 0) s_pick[warp] = pick;
    const int pr = active[pick];
    const uint32_t pw = grid[pr];
    const int prx = pr % SYN_R, pry = (pr / SYN_R) % SYN_R, prz = pr / (SYN_R * SYN_R);
    const int BX = (prx + ox) * SYN_Q + static_cast<int>(pw & 1023u);
    const int BY = (pry + oy) * SYN_Q + static_cast<int>((pw >> 10) & 1023u);
    const int BZ = (prz - 2) * SYN_Q + static_cast<int>((pw >> 20) & 1023u);
    bool valid = false;
    int X = 0, Y = 0, Z = 0, rb = 0;
    if (lane < SYN_K) {
      const float u = uf(r.x);
      const float ct = uf(r.y) * 2.0f - 1.0f;
      const float st = sqrtf(fmaxf(1.0f - ct * ct, 0.0f));
      float sp, cp;
      sincospif(uf(r.z) * 2.0f, &sp, &cp);
      const float rad = cbrtf(7.0f * u + 1.0f) * 1.7320508075688772f;  // r = sqrt(3) cells
      const float fx = static_cast<float>(BX) * (1.0f / SYN_Q) + rad * st * cp;
      const float fy = static_cast<float>(BY) * (1.0f / SYN_Q) + rad * st * sp;
      const float fz = static_cast<float>(BZ) * (1.0f / SYN_Q) + rad * ct;
      if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f) {
        X = static_cast<int>(floorf(fx * SYN_Q));
        Y = static_cast<int>(floorf(fy * SYN_Q));
        Z = static_cast<int>(floorf(fz * SYN_Q));
        if (X < static_cast<int>(t.XW) && Y < static_cast<int>(t.YW) && Z < static_cast<int>(t.ZW)) {
          const int cx = X >> 10, cy = Y >> 10, cz = Z >> 10;
          const int rx = cx - ox, ry = cy - oy, rz = cz + 2;
          // The neighbourhood must lie inside the staged region (it does for candidates within 2r
          // of a point of the column); a candidate that fails the check is rejected.
          if (cx >= x0 - SYN_SPILL && cx < x1 + SYN_SPILL && cy >= y0 - SYN_SPILL && cy < y1 + SYN_SPILL &&
              index_ok(rx >= 2 && rx <= SYN_R - 3 && ry >= 2 && ry <= SYN_R - 3 && rz >= 2 && rz <= nz - 3, err,
                       SITE_SYN_REGION, static_cast<uint32_t>(rx | (ry << 8) | (rz << 16)), blockIdx.x)) {
            rb = (rz * SYN_R + ry) * SYN_R + rx;
            valid = syn_near_free(grid, rb, X & 1023, Y & 1023, Z & 1023);
          }
        }
      }
    }
    unsigned rest;
    const bool first = syn_outer_free(grid, s_outer, valid, rb, X & 1023, Y & 1023, Z & 1023, lane, rest);
    const unsigned vm = __ballot_sync(0xffffffffu, first);
    if (first || ((rest >> lane) & 1u)) {
      s_cx[warp][lane] = X;
      s_cy[warp][lane] = Y;
      s_cz[warp][lane] = Z;
    }
    if (lane == 0) {
      s_vmask[warp] = vm;
      s_rmask[warp] = rest;
    }
    __syncthreads();
    if (warp == 0) {
      // The round's steps in warp order, exactly as if they ran one after another: warp w keeps its
      // first candidate (lane order) that is free in the grid and at least r from the points
      // accepted for warps < w; with none left, its point retires.
      //
      // Lane w speaks for warp w and holds its winner (first grid-free candidate).  That order keeps
      // a winner unless it lies within r of a point accepted for an earlier warp, so the warps keep
      // their winners in runs up to the next warp whose winner conflicts; only that warp searches
      // its other candidates against the points accepted so far.  Conflicts between winners come
      // from shuffles; a point kept instead of a winner is tested against the later winners once.
      int fw = -1, PX = 0, PY = 0, PZ = 0;
      if (lane < SYN_WARPS) {
        const unsigned m = s_vmask[lane];
        if (m) {
          fw = __ffs(m) - 1;
          PX = s_cx[lane][fw];
          PY = s_cy[lane][fw];
          PZ = s_cz[lane][fw];
        }
      }
      unsigned cm = 0;  // bit u: this lane's winner conflicts with warp u's (u < lane)
#pragma unroll
      for (int u = 0; u < SYN_WARPS - 1; ++u) {
        const int ux = __shfl_sync(0xffffffffu, PX, u), uy = __shfl_sync(0xffffffffu, PY, u);
        const int uz = __shfl_sync(0xffffffffu, PZ, u), uf = __shfl_sync(0xffffffffu, fw, u);
        if (u < lane && fw >= 0 && uf >= 0) {
          const int ex = PX - ux, ey = PY - uy, ez = PZ - uz;
          if (ex * ex + ey * ey + ez * ez < SYN_R2X) cm |= 1u << u;
        }
      }
      const unsigned has = __ballot_sync(0xffffffffu, fw >= 0);  // warps with a winner
      unsigned accw = 0, acc = 0;  // warps that keep their winner; warps that keep a point
      bool near = false;           // this lane's winner lies within r of a point kept instead of a winner
      for (int cur = 0; cur < SYN_WARPS;) {
        // A warp from cur on keeps its winner unless it conflicts with a kept point; up to the first
        // such warp, every warp with a winner keeps it.
        const unsigned from = ~((1u << cur) - 1u);
        const bool bad = lane >= cur && fw >= 0 &&
                         (near || (cm & (accw | (has & from & ((1u << lane) - 1u)))) != 0u);
        const unsigned bm = __ballot_sync(0xffffffffu, bad);
        const int wb = bm ? __ffs(bm) - 1 : SYN_WARPS;
        const unsigned run = has & from & ((1u << wb) - 1u);
        accw |= run;
        acc |= run;
        if (wb == SYN_WARPS) break;
        // Warp wb: its first valid candidate at least r from every point kept for warps < wb.  Its
        // untested candidates take the outer test here, in lane order, until one passes (the grid
        // is as the candidate phase saw it: the round commits after it is resolved).
        const unsigned m = s_vmask[wb], mr = s_rmask[wb];
        bool ok = ((m | mr) >> lane) & 1u;
        int X = 0, Y = 0, Z = 0;
        if (ok) {
          X = s_cx[wb][lane];
          Y = s_cy[wb][lane];
          Z = s_cz[wb][lane];
        }
#pragma unroll
        for (int u = 0; u < SYN_WARPS - 1; ++u) {
          const int ux = __shfl_sync(0xffffffffu, PX, u), uy = __shfl_sync(0xffffffffu, PY, u);
          const int uz = __shfl_sync(0xffffffffu, PZ, u);
          if ((acc >> u) & 1u) {
            const int ex = X - ux, ey = Y - uy, ez = Z - uz;
            if (ex * ex + ey * ey + ez * ez < SYN_R2X) ok = false;
          }
        }
        unsigned okm = __ballot_sync(0xffffffffu, ok);
        int c = -1;
        while (okm) {
          const int l = __ffs(okm) - 1;
          okm &= okm - 1;
          if ((m >> l) & 1u) {
            c = l;
            break;
          }
          const int lx_ = __shfl_sync(0xffffffffu, X, l), ly_ = __shfl_sync(0xffffffffu, Y, l);
          const int lz_ = __shfl_sync(0xffffffffu, Z, l);
          const int cb = (((lz_ >> 10) + 2) * SYN_R + ((ly_ >> 10) - oy)) * SYN_R + ((lx_ >> 10) - ox);
          if (!syn_outer_hit(grid, s_outer, cb, lx_ & 1023, ly_ & 1023, lz_ & 1023, lane)) {
            c = l;
            break;
          }
        }
        if (c >= 0) {
          const int qx = __shfl_sync(0xffffffffu, X, c), qy = __shfl_sync(0xffffffffu, Y, c);
          const int qz = __shfl_sync(0xffffffffu, Z, c);
          acc |= 1u << wb;
          if (lane == wb) {
            PX = qx;
            PY = qy;
            PZ = qz;
          } else if (lane > wb && fw >= 0) {
            const int ex = PX - qx, ey = PY - qy, ez = PZ - qz;
            if (ex * ex + ey * ey + ez * ez < SYN_R2X) near = true;
          }
        }
        cur = wb + 1;
      }
      // Commit the kept points, appending to the active list in warp order.
      bool inside = false, committed = false;
      int cridx = 0;
      if (lane < SYN_WARPS && ((acc >> lane) & 1u)) {
        const int ccx = PX >> 10, ccy = PY >> 10, ccz = PZ >> 10;
        const int rx = ccx - ox, ry = ccy - oy, rz = ccz + 2;
        if (index_ok(rx >= 0 && rx < SYN_R && ry >= 0 && ry < SYN_R && rz >= 0 && rz < nz, err, SITE_SYN_COMMIT,
                     static_cast<uint32_t>(rx | (ry << 8) | (rz << 16)), blockIdx.x)) {
          cridx = (rz * SYN_R + ry) * SYN_R + rx;
          grid[cridx] = syn_word(PX, PY, PZ);
          committed = true;
          inside = ccx >= x0 && ccx < x1 && ccy >= y0 && ccy < y1;
        }
      }
      const unsigned im = __ballot_sync(0xffffffffu, inside);
      const int nbase = s_nact;
      if (inside) {
        const int pos = nbase + __popc(im & ((1u << lane) - 1u));
        if (index_ok(pos < acap, err, SITE_SYN_ACTIVE, pos, blockIdx.x)) active[pos] = static_cast<uint16_t>(cridx);
      }
      const unsigned cmm = __ballot_sync(0xffffffffu, committed);
      const int n0 = min(nbase + __popc(im), acap);
      __syncwarp();  // the appended entries are visible to the retirement below
      // Retire the points of failed steps, each once, as if removed one after another in descending
      // list order, each by moving the list's current last entry into its place (a swap-remove).
      // The removal of rank k takes the entry then at n0 - 1 - k; when that position was itself
      // refilled by an earlier removal, its entry is the one that removal took, so each removal
      // follows that chain (pointer jumping over the ranks) to an original position.
      const bool mine = lane < SYN_WARPS && !((acc >> lane) & 1u);
      const int mypick = lane < SYN_WARPS ? s_pick[lane] : -1;
      const unsigned peers = __match_any_sync(0xffffffffu, mine ? mypick : -1 - lane);
      const bool first = mine && lane == __ffs(peers) - 1;
      const unsigned dm = __ballot_sync(0xffffffffu, first);
      int rank = 0;
#pragma unroll
      for (int w2 = 0; w2 < SYN_WARPS; ++w2) {
        const int p2 = __shfl_sync(0xffffffffu, mypick, w2);
        if (((dm >> w2) & 1u) && p2 > mypick) ++rank;
      }
      int src = n0 - 1 - rank, ptr = -1;
#pragma unroll
      for (int w2 = 0; w2 < SYN_WARPS; ++w2) {
        const int p2 = __shfl_sync(0xffffffffu, mypick, w2);
        if (((dm >> w2) & 1u) && w2 != lane && p2 == src) ptr = w2;
      }
      if (!first) ptr = -1;
#pragma unroll
      for (int hop = 1; hop < SYN_WARPS; hop <<= 1) {  // chains are shorter than SYN_WARPS
        const int at = ptr < 0 ? lane : ptr;
        const int ps = __shfl_sync(0xffffffffu, src, at), pp = __shfl_sync(0xffffffffu, ptr, at);
        if (ptr >= 0) {
          src = ps;
          ptr = pp;
        }
      }
      uint16_t moved = 0;
      if (first && index_ok(src >= 0 && src < n0, err, SITE_SYN_ACTIVE, src, blockIdx.x)) moved = active[src];
      __syncwarp();
      if (first && src >= 0 && src < n0) active[mypick] = moved;
      if (lane == 0) {
        s_nact = n0 - __popc(dm);
        s_ncom += __popc(cmm);
      }
    }
  }
  __syncthreads();
  // Write back the column and its spill zone.
  for (int i = tid; i < ncell; i += blockDim.x) {
    const int rx = i % SYN_R, ry = (i / SYN_R) % SYN_R, rz = i / (SYN_R * SYN_R);
    if (rx < 2 || ry < 2 || rx >= SYN_R - 2 || ry >= SYN_R - 2) continue;
    const int gx = ox + rx, gy = oy + ry, gz = rz - 2;
    if (gx >= 0 && gy >= 0 && gz >= 0 && gx < static_cast<int>(t.gw) && gy < static_cast<int>(t.gh) && gz < gd)
      tc[(static_cast<size_t>(gz) * t.gh + gy) * t.gw + gx] = grid[i];
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    if (s_ncom) atomicAdd(npts + lo, static_cast<uint32_t>(s_ncom));
    atomicExch(done + blockIdx.x, 1u);
  }
}

// Independent deletion down to the Bridson-expected count: each point goes with probability p,
// drawn from the Philox block of its cell.  blockIdx.y is the tile (the points per tile were
// counted by k_bridson).  Each warp reads 32 cells at a time and queues the occupied ones; the
// draws run once 32 are queued, with every lane busy.
constexpr int THIN_T = 256;
__global__ void __launch_bounds__(THIN_T) k_thin(const SynthTile* __restrict__ tiles, uint32_t* __restrict__ cells,
                                                 const uint32_t* npts) {
  const SynthTile& t = tiles[blockIdx.y];
  const uint32_t n = npts[blockIdx.y];
  if (n <= t.target) return;
  const float p = 1.0f - static_cast<float>(t.target) / static_cast<float>(n);
  const uint32_t nc = t.gw * t.gh * t.gd;
  uint32_t* tc = cells + t.cell_base;
  const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
  __shared__ uint32_t s_q[THIN_T / 32][64];
  uint32_t* q = s_q[threadIdx.x >> 5];
  uint32_t fill = 0;  // the same in every lane of the warp
  auto thin = [&](uint32_t lin) {
    if (uf(philox(lin, 0, 0, TAG_THIN, t.k0, t.k1).x) < p) tc[lin] = 0;
  };
  const uint32_t warps = gridDim.x * (THIN_T / 32);
  for (uint32_t base = (blockIdx.x * THIN_T + threadIdx.x - lane); base < nc; base += warps * 32) {
    const uint32_t lin = base + lane;
    const bool occ = lin < nc && (tc[lin] & OCC);
    const unsigned m = __ballot_sync(0xffffffffu, occ);
    if (occ) q[fill + __popc(m & lt)] = lin;
    fill += __popc(m);
    __syncwarp();
    if (fill >= 32) {
      const uint32_t mine = q[lane];
      const uint32_t rest = fill - 32;
      const uint32_t moved = lane < rest ? q[32 + lane] : 0u;
      __syncwarp();
      if (lane < rest) q[lane] = moved;
      fill = rest;
      __syncwarp();
      thin(mine);
    }
  }
  if (lane < fill) thin(q[lane]);
}

// Cell of compaction slot sl: the brick (2D Morton over the high x, y bits) in the bits above
// 3 * brick_bits, the cell inside it (3D Morton, x lowest) below.
__device__ __forceinline__ void slot_cell(const SynthTile& t, uint32_t sl, uint32_t& x, uint32_t& y, uint32_t& z) {
  const uint32_t L = t.brick_bits;
  const uint32_t lo = sl & ((1u << (3 * L)) - 1u), hi = sl >> (3 * L);
  x = (morton2_compact(hi) << L) | morton3_compact(lo);
  y = (morton2_compact(hi >> 1) << L) | morton3_compact(lo >> 1);
  z = morton3_compact(lo >> 2);
}

// Points per brick (the compaction unit): one block per brick counts the occupied cells of its
// region, read row by row.  blockIdx.y is the tile.
__global__ void k_brick_count(const SynthTile* __restrict__ tiles, const uint32_t* __restrict__ cells,
                              uint32_t* counts) {
  const SynthTile& t = tiles[blockIdx.y];
  const uint32_t L = t.brick_bits, E = 1u << L;
  const uint32_t nbricks = 1u << (2 * t.slot_bits);
  const uint32_t* tc = cells + t.cell_base;
  __shared__ uint32_t s_sum[32];
  for (uint32_t b = blockIdx.x; b < nbricks; b += gridDim.x) {
    const uint32_t xb = morton2_compact(b) << L, yb = morton2_compact(b >> 1) << L;
    const uint32_t ex = xb < t.gw ? min(E, t.gw - xb) : 0u, ey = yb < t.gh ? min(E, t.gh - yb) : 0u;
    const uint32_t ez = min(E, t.gd), n = ex * ey * ez;
    uint32_t c = 0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const uint32_t x = xb + i % ex, y = yb + (i / ex) % ey, z = i / (ex * ey);
      c += (tc[(static_cast<size_t>(z) * t.gh + y) * t.gw + x] & OCC) ? 1u : 0u;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t tot = 0;
      for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) tot += s_sum[w];
      counts[t.slot_base + b] = tot;
    }
    __syncthreads();
  }
}

// Crystal k of a tile at compaction slot sl (cell x, y, z): position from the fixed-point cell
// word, attributes from the tile's Philox stream keyed by the cell (emulsion.rs:162-200).
__device__ __forceinline__ void emit_crystal(const SynthTile& t, const uint32_t* __restrict__ cells, uint32_t sl,
                                             uint32_t x, uint32_t y, uint32_t z, uint32_t k, float4* A, float4* Q,
                                             float4* D, uint64_t* keys) {
  const uint32_t lin = (z * t.gh + y) * t.gw + x;
  const uint32_t w = cells[t.cell_base + lin];
  const float px = static_cast<float>(static_cast<int>(x) * SYN_Q + static_cast<int>(w & 1023u)) * (t.cell / SYN_Q);
  const float py = static_cast<float>(static_cast<int>(y) * SYN_Q + static_cast<int>((w >> 10) & 1023u)) * (t.cell / SYN_Q);
  const float pz = static_cast<float>(static_cast<int>(z) * SYN_Q + static_cast<int>((w >> 20) & 1023u)) * (t.cell / SYN_Q);
  const P4 r0 = philox(lin, 0, 0, TAG_ATTR, t.k0, t.k1);
  const P4 r1 = philox(lin, 1, 0, TAG_ATTR, t.k0, t.k1);
  // Two normals from one Box-Muller pair: radius (log-normal) and sensitivity.
  const float bm = sqrtf(-2.0f * logf(1.0f - uf(r0.x)));
  float s2, c2;
  sincospif(2.0f * uf(r0.y), &s2, &c2);
  const float radius = fminf(fmaxf(expf(t.mu + t.sg * bm * c2), 0.15f), t.rmax);
  const float sens = fmaxf(t.base_sens + 0.15f * bm * s2, 0.1f);
  float4 q, d;
  if (t.morph == 1) {
    // Tabular: thickness r / AR (>= 0.05), tilt +-0.17 rad about a random in-plane axis.
    const float ht = fmaxf(radius / t.aspect, 0.05f);
    const float tilt = uf(r0.z) * 0.34f - 0.17f;
    float ax = uf(r0.w) * 2.0f - 1.0f, ay = uf(r1.x) * 2.0f - 1.0f;
    const float n = rsqrtf(fmaxf(ax * ax + ay * ay, 1e-30f));
    ax *= n;
    ay *= n;
    float sh, ch;
    sincosf(0.5f * tilt, &sh, &ch);
    q = make_float4(ax * sh, ay * sh, 0.0f, ch);
    d = make_float4(radius, radius, ht, __int_as_float(1));
  } else {
    // Cubic / octahedral: UnitQuaternion::from_euler_angles(2 pi u1, pi u2, 2 pi u3).
    float sr, cr, sp, cp, sy, cy;
    sincospif(uf(r0.z), &sr, &cr);        // roll / 2 = pi u1
    sincospif(0.5f * uf(r0.w), &sp, &cp); // pitch / 2 = pi u2 / 2
    sincospif(uf(r1.x), &sy, &cy);        // yaw / 2 = pi u3
    q = make_float4(sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy, cr * cp * sy - sr * sp * cy,
                    cr * cp * cy + sr * sp * sy);
    d = make_float4(radius, radius, radius, __int_as_float(t.morph));
  }
  const unsigned long long o = t.cbase + k;
  A[o] = make_float4(px, py, pz, sens);
  Q[o] = q;
  D[o] = d;
  keys[o] = sl;
}

// The crystals of each brick in slot order (slot_cell): the brick's slots are walked in chunks of
// the block, a block-wide prefix sum of the occupied ones numbers them after the points of the
// earlier bricks (scan: exclusive sum of k_brick_count).  About one cell in nine holds a point,
// so the numbered crystals are queued in shared memory and made once the queue holds a block's
// worth, with every lane busy.  blockIdx.y is the tile.
constexpr int EMIT_T = 256;
__global__ void __launch_bounds__(EMIT_T) k_emit(const SynthTile* __restrict__ tiles,
                                                 const uint32_t* __restrict__ cells,
                                                 const uint32_t* __restrict__ scan, float4* A, float4* Q,
                                                 float4* D, uint64_t* keys, uint32_t* err) {
  const SynthTile& t = tiles[blockIdx.y];
  const uint32_t L = t.brick_bits;
  const uint32_t nbricks = 1u << (2 * t.slot_bits), per = 1u << (3 * L);
  const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr uint32_t NW = EMIT_T / 32;
  __shared__ uint32_t s_w[NW + 1];
  __shared__ uint32_t s_k[2 * EMIT_T], s_sl[2 * EMIT_T];  // queued crystals: number and slot
  uint32_t fill = 0;                                      // queue length (the same in every thread)
  auto drain = [&]() {
    for (uint32_t i = threadIdx.x; i < fill; i += EMIT_T) {
      const uint32_t sl = s_sl[i], k = s_k[i];
      if (k >= t.ccap) continue;  // past the tile's capacity (flagged when queued)
      uint32_t x, y, z;
      slot_cell(t, sl, x, y, z);
      emit_crystal(t, cells, sl, x, y, z, k, A, Q, D, keys);
    }
    fill = 0;
    __syncthreads();
  };
  for (uint32_t b = blockIdx.x; b < nbricks; b += gridDim.x) {
    const unsigned long long bi = t.slot_base + b;
    if (scan[bi + 1] == scan[bi]) continue;  // block-uniform
    uint32_t k0 = scan[bi] - scan[t.slot_base];
    const uint32_t xb = morton2_compact(b) << L, yb = morton2_compact(b >> 1) << L;
    for (uint32_t c0 = 0; c0 < per; c0 += EMIT_T) {
      const uint32_t lo = c0 + threadIdx.x;
      const uint32_t x = xb | morton3_compact(lo), y = yb | morton3_compact(lo >> 1), z = morton3_compact(lo >> 2);
      const bool occ = lo < per && x < t.gw && y < t.gh && z < t.gd &&
                       (cells[t.cell_base + (static_cast<size_t>(z) * t.gh + y) * t.gw + x] & OCC);
      const unsigned m = __ballot_sync(0xffffffffu, occ);
      if (lane == 0) s_w[warp] = __popc(m);
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (uint32_t w = 0; w < NW; ++w) {
          const uint32_t v = s_w[w];
          s_w[w] = acc;
          acc += v;
        }
        s_w[NW] = acc;
      }
      __syncthreads();
      if (occ) {
        const uint32_t r = s_w[warp] + __popc(m & ((1u << lane) - 1u));
        const uint32_t k = k0 + r;
        if (k >= t.ccap) atomicOr(err, ERR_LIST_OVERFLOW);
        s_k[fill + r] = k;
        s_sl[fill + r] = (b << (3 * L)) | lo;
      }
      const uint32_t got = s_w[NW];
      k0 += got;
      fill += got;
      __syncthreads();
      if (fill >= EMIT_T) drain();
    }
  }
  drain();
}

}  // namespace fg

namespace fg {

size_t bridson_smem(int gdmax);

// Host wrappers (launch on `st`; all buffers preallocated so the sequence can be graph-captured).
// cols[c] columns of class c; done holds one flag per column (zeroed here).
void launch_bridson(const SynthTile* tiles, int ntiles, const unsigned cols[4], int gdmax, uint32_t* cells,
                    uint32_t* npts, uint32_t* done, uint32_t* err, cudaStream_t st, uint32_t wait_limit,
                    const uint32_t* probe) {
  const unsigned total = cols[0] + cols[1] + cols[2] + cols[3];
  if (total == 0) return;
  const int nz = gdmax + 4;
  const size_t smem = bridson_smem(gdmax);
  FG_CUDA(cudaMemsetAsync(done, 0, total * sizeof(uint32_t), st));
  FG_CUDA(cudaFuncSetAttribute(k_bridson, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  const uint4 cb = make_uint4(0u, cols[0], cols[0] + cols[1], cols[0] + cols[1] + cols[2]);
  k_bridson<<<total, SYN_WARPS * 32, smem, st>>>(tiles, ntiles, cb, nz, cells, npts, done, err,
                                                  wait_limit ? wait_limit : (1u << 22), probe);
  FG_CUDA(cudaGetLastError());
}

size_t bridson_smem(int gdmax) {
  return static_cast<size_t>(SYN_R) * SYN_R * (gdmax + 4) * sizeof(uint32_t) +
         static_cast<size_t>(SYN_B) * SYN_B * gdmax * sizeof(uint16_t);
}

// Per-tile grids (blockIdx.y is the tile): max_cells and max_bricks are the largest tile's.
void launch_synth_post(const SynthTile* tiles, int ntiles, unsigned long long max_cells, unsigned long long max_bricks,
                       uint32_t* cells, uint32_t* npts, uint32_t* counts, cudaStream_t st) {
  if (ntiles == 0) return;
  FG_REQUIRE(ntiles <= 65535, "too many tiles for one launch");
  const unsigned bc = static_cast<unsigned>(std::min<unsigned long long>(std::max(grid_for(max_cells, 256), 1u), 1024));
  const unsigned bb = static_cast<unsigned>(std::min<unsigned long long>(std::max(max_bricks, 1ull), 4096));
  k_thin<<<dim3(bc, ntiles), THIN_T, 0, st>>>(tiles, cells, npts);
  k_brick_count<<<dim3(bb, ntiles), 256, 0, st>>>(tiles, cells, counts);
  FG_CUDA(cudaGetLastError());
}

void launch_emit(const SynthTile* tiles, int ntiles, unsigned long long max_bricks, const uint32_t* cells,
                 const uint32_t* scan, float4* A, float4* Q, float4* D, uint64_t* keys, uint32_t* err,
                 cudaStream_t st) {
  if (ntiles == 0) return;
  FG_REQUIRE(ntiles <= 65535, "too many tiles for one launch");
  const unsigned bb = static_cast<unsigned>(std::min<unsigned long long>(std::max(max_bricks, 1ull), 4096));
  k_emit<<<dim3(bb, ntiles), EMIT_T, 0, st>>>(tiles, cells, scan, A, Q, D, keys, err);
  FG_CUDA(cudaGetLastError());
}

}  // namespace fg
