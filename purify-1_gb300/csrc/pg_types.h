// Plain-old-data types shared by the host planner and the device kernels.
//
// Layout in HBM of one coverage (the measurement set of one operator), all in
// "plan order" (visibilities sorted by uv tile, then by base cell):
//   vis_t    [M]   real2   fractional offsets (t_u, t_v) in [0, 1) of each
//                          visibility inside its base cell, computed in FP64
//   vis_w    [M]   complex weight x (-1)^(k_u + k_v)  (the phase sign of the
//                          reference's exp(-2 pi i (k_u + k_v)/2) folded in)
//   vis_perm [M]   int32   index of the visibility in the caller's order
//   items    [NI]  int2    work items: {first visibility, packed cell+count}
//   tasks    [NT]  Task    CTA work units: a tile and a range of 32-item batches
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define PG_HD __host__ __device__
#else
#define PG_HD
#endif

namespace pg {

// Status codes of the C-ABI (mirrored in include/purify_gb300.h).
enum Status : int {
  kOk = 0,
  kInvalidArgument = 1,
  kUnsupported = 2,
  kCudaError = 3,
  kOutOfMemory = 4,
  kNormNotPositive = 5,
  kRejected = 6,
  kTimeout = 7,
  kInternal = 8,
};

// Kernel identifiers in the order of the reference's kernels::kernel enum.
enum KernelId : int { kKB = 0, kGauss = 1, kBox = 2, kPSWF = 3, kKBMin = 4, kGaussAlt = 5 };

// Largest separable support handled by the plain (non w-projection) kernels.
constexpr int kMaxJ = 8;
// Largest support whose items may group 2 x 2 base cells (complex<float>
// only: the (J + 1)^2 register block must stay in registers).
constexpr int kMaxGroupJ = 6;
// Largest number of sub-segments per tap of a piecewise kernel polynomial.
constexpr int kMaxSub = 4;
// Polynomial coefficient counts (degree + 1) per precision.
constexpr int kCoefF32 = 9;
constexpr int kCoefF64 = 17;
// Tile edge (in grid cells) of the uv tiling.
constexpr int kTile = 32;
// Warps of a column-walk task of G^H; warp w takes base-cell columns
// [w W / kWalkWarps, (w + 1) W / kWalkWarps) of a tile W <= 32 wide.
constexpr int kWalkWarps = 4;
// Lanes per batch: every batch holds 32 work items, one per lane.
constexpr int kBatch = 32;
// Most batches one CTA task may hold (its headers are staged in shared memory).
constexpr int kMaxTaskBatches = 64;
// Grids up to this many bytes (as complex<float>) launch their tasks longest
// first; larger ones in spatial order (see plan.h).
constexpr int64_t kLptGridBytes = int64_t(64) << 20;

// One CTA work unit.  A tile is the rectangle [P, P+H) x [Q, Q+W) of base
// cells; its grid window is (H + J - 1) x (W + J - 1) cells starting at (P, Q),
// wrapped periodically.
struct Task {
  int32_t P, Q, H, W;
  int32_t batch_begin, batch_end;  // [begin, end) in units of 32-item batches
  int32_t tile;                    // tile id (tile_row * ntu + tile_col)
  int32_t channel;                 // operator of a grouped (multi-channel) launch, else 0
};

// A run of consecutive visibilities (plan order) of one w-projection task
// whose row factors, [fbegin, fend) in complex values, are staged in shared
// memory together.
struct WChunk {
  int64_t fbegin, fend;
  int32_t vis_begin, vis_end;
};
// Bounds of a w-projection chunk: visibilities, and factor values (raised to
// 6 Smax when one row needs more).
constexpr int kWChunkVis = 64;
constexpr int kWChunkValues = 1024;

// Work item encoding: .x = first visibility (plan order), .y = lp | lq << 8 |
// count << 16 with (lp, lq) the base cell relative to the tile origin.  An
// item with count 0 is padding.
PG_HD inline int item_lp(int y) { return y & 0xff; }
PG_HD inline int item_lq(int y) { return (y >> 8) & 0xff; }
PG_HD inline int item_count(int y) { return (y >> 16) & 0xffff; }
inline int item_pack(int lp, int lq, int count) { return lp | (lq << 8) | (count << 16); }

// Piecewise-polynomial kernel state: for tap j (0-based) and sub-segment s,
// P_{j,s}(x) = sum_k c[j][s][k] x^k with x = 2 (t nsub - s) - 1 in [-1, 1)
// approximates (-1)^j * kernel(t + J/2 - 1 - j).  Coefficients are fitted in
// FP64 on the host; the device evaluates them by Horner's rule.
template <typename real, int NCOEF>
struct PolyAxis {
  real c[kMaxJ][kMaxSub][NCOEF];
};

template <typename real>
struct PolyCount;
template <>
struct PolyCount<float> {
  static constexpr int value = kCoefF32;
};
template <>
struct PolyCount<double> {
  static constexpr int value = kCoefF64;
};

template <typename real>
struct PolyTable {
  PolyAxis<real, PolyCount<real>::value> u, v;
  int32_t nsub_u, nsub_v;
};

}  // namespace pg
