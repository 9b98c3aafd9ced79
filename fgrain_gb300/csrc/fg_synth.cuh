// Device crystal synthesis (emulsion.rs:155-220, poisson.rs:14-132).
//
// Bridson's sampler is sequential.  On the device the tile's cell grid (cell = r_min / sqrt(3),
// at most one point per cell, as poisson.rs:25-31) is cut into columns of SYN_B x SYN_B cells that
// span the full depth.  Columns are processed in four colour classes (column x and y parity);
// columns of one class are a column apart, so they never touch the same cells.  Each column runs
// Bridson (k = 30 candidates in the shell [r, 2r], first valid candidate wins) from the points
// already inside it (spilled in by earlier classes) or from one random seed; accepted points may
// lie up to SYN_SPILL cells outside the column (the rest of the shell is left to the neighbouring
// columns of later classes).  Each round, every warp of the column's CTA takes a Bridson step on a
// randomly picked active point, one candidate per lane; then one warp resolves the steps in warp
// order exactly as if they had run one after another (a step keeps its first candidate that is
// also at least r from the points accepted for earlier warps, else its point retires).
// Positions are fixed point (1/1024 of a cell) so every distance test is exact integer arithmetic.
//
// Bridson started from many seeds packs denser than from one (0.3-0.9 % per tile on a 1024^2
// tri-x image at supersample 2; 1.2-1.7 % with a spill of two cells, -1.3 % with none: the
// columns' walls then leave gaps), so each tile is then thinned (independent deletion) to the
// count Bridson yields on the same box:
// rho r^3 = 0.57793 + 0.11307 r (2/W + 2/H + 2/D), fitted to the reference sampler over box
// sizes 27-160 um and depths 6-20 um (residuals within 0.12 %).
#pragma once
#include "fg_device.cuh"

namespace fg {

constexpr int SYN_B = 8;         // column edge in cells
constexpr int SYN_SPILL = 1;     // cells an accepted point may lie outside its column
constexpr int SYN_HALO = SYN_SPILL + 2;      // + the reach of the neighbourhood test
constexpr int SYN_R = SYN_B + 2 * SYN_HALO;  // staged region edge
// Columns of one colour class are one column apart: what one writes (its spill zone) must not
// reach what another reads (its halo).
static_assert(SYN_SPILL + SYN_HALO <= SYN_B, "colour classes would overlap");
constexpr int SYN_WARPS = 8;
constexpr int SYN_K = 30;        // Bridson's k
constexpr int32_t SYN_Q = 1024;  // fixed-point steps per cell
constexpr int32_t SYN_R2 = 3 * SYN_Q * SYN_Q;  // r^2 with r = sqrt(3) cells
// Exclusion radius squared of the sampler: r^2 plus 128 units^2 (2e-5 r), so that two points kept
// at the smallest allowed distance are still r_min apart after their positions are rounded to
// float (about 1e-5 um at 100 um).
constexpr int32_t SYN_R2X = SYN_R2 + 128;
constexpr uint32_t OCC = 0x80000000u;

__host__ __device__ inline double bridson_density(double W, double H, double D, double r) {
  return (0.57793168 + 0.11306788 * r * (2.0 / W + 2.0 / H + 2.0 / D)) / (r * r * r);
}

struct __align__(16) SynthTile {
  unsigned long long cell_base;  // first cell of this tile in the batch grid
  unsigned long long slot_base;  // first brick of this tile in the batch's brick counts
  unsigned long long cbase;      // first crystal slot
  uint32_t gw, gh, gd;           // cell grid
  uint32_t nbx, nby;             // columns per axis
  uint32_t XW, YW, ZW;           // exclusive bounds of fixed-point coordinates
  // Compaction slots in brick order: bricks of 2^brick_bits cells per axis (brick_bits covers the
  // depth), bricks in 2D Morton order (slot_bits per axis), cells in 3D Morton order inside a
  // brick.  Slot order is crystal order and the LBVH key, so the tree's lower levels group
  // compact 3D blocks of crystals, not full-depth columns.
  uint32_t slot_bits, slots;     // slots = 4^slot_bits * 8^brick_bits
  uint32_t brick_bits;
  uint32_t ccap;                 // crystal capacity
  uint32_t target;               // Bridson-expected crystal count
  uint32_t k0, k1;               // synthesis key (tile seed)
  uint32_t col_base[5];          // first global column of each colour class (prefix over tiles)
  float cell;                    // cell edge (um)
  // Crystal attributes (emulsion.rs:162-200).
  float mu, sg;                  // log-normal radius parameters
  float rmax;                    // radius clamp top (0.48 r_min)
  float base_sens;
  float aspect;                  // tabular aspect ratio
  int morph;
};

}  // namespace fg
