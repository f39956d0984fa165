// Coverage planning (host, FP64): everything about a set of visibilities that
// does not change between applies of the operator.
//
// Visibilities are sorted by uv tile and base cell, grouped into work items
// (one base cell, up to K visibilities) and packed into batches of 32 items,
// one item per lane, no two items of a batch on the same base cell, items on
// the lanes of their shared-memory bank classes where free (see
// Plan::win_stride).  Each
// batch owns 32 * kmax consecutive "slots" (kmax = its largest item): lane l's
// k-th visibility sits in slot base + 32 k + l, so a warp that walks k reads
// 256 contiguous bytes per access and every lane runs the same loop.  Lanes
// whose item is shorter than kmax own null slots (no visibility).
#pragma once
#include <complex>
#include <cstdint>
#include <vector>

#include "pg_types.h"

namespace pg {

struct PlanRequest {
  const double *u = nullptr;  // M coordinates in grid pixels
  const double *v = nullptr;
  const std::complex<double> *weights = nullptr;  // M weights, or null for ones
  int64_t M = 0;
  int Nu = 0, Nv = 0;  // grid width (u, fastest) and height (v)
  int Ju = 4, Jv = 4;  // taps per axis
  int tile = kTile;
  int max_per_item = 16;         // visibilities of one cell handled by one lane
  // Cells of a work item (group code): 1 = one base cell; 2 = an aligned
  // 2 x 2 group of base cells of its tile (anchored at even local row and
  // column), whose visibilities share one (J + 1) x (J + 1) register block;
  // 3 = an aligned pair of adjacent cells of a row (anchored at an even
  // local column), a J x (J + 1) block.  A visibility carries its cell
  // inside the group in the integer part of its fractions (t_u + dx,
  // t_v + dy with dx, dy in {0, 1}).
  int group = 1;
  // Most items of one bank class per batch (0: the default, see plan.cpp).
  int class_cap = 0;
  int max_batches_per_task = kMaxTaskBatches;
  int64_t max_slots_per_task = 16384;
  // Warps of the CTAs that will run the plan: the kernels deal a task's
  // batches round-robin (batch i to warp i mod warps), and the planner
  // orders each task's batches so that this dealing balances the warps.
  int warps = 4;
};

// Tiling of one grid axis: tile b covers [start[b], start[b + 1]).
struct AxisTiling {
  int n = 0;
  std::vector<int32_t> start;  // n + 1 entries
  std::vector<int32_t> of;     // axis length entries: tile index of each cell
};

struct Plan {
  int64_t M = 0;  // visibilities
  int64_t S = 0;  // slots (>= M)
  int Nu = 0, Nv = 0, Ju = 0, Jv = 0;
  AxisTiling tu, tv;  // tilings of the u (columns) and v (rows) axes
  // True when every weight is exactly 1: the weight stream is then replaced
  // by the phase sign alone.
  bool unit_weights = true;
  // per slot
  std::vector<double> frac_u, frac_v;        // t + d in [0, group); 0 for null slots
  std::vector<uint8_t> flip;                 // (-1)^(k_u + k_v) == -1
  std::vector<std::complex<double>> weight;  // weight with the sign folded in (empty when unit)
  std::vector<int32_t> slot_user;            // caller index, -1 for null slots
  // per visibility
  std::vector<int32_t> user_slot;  // caller index -> slot
  // per batch
  std::vector<int32_t> batch_base, batch_kmax;
  std::vector<int32_t> lane_code;  // batch * 32 + lane -> item_pack(lp, lq, count)
  std::vector<Task> tasks;
  // Launch order of the tasks: by decreasing slot count (longest first) when
  // the grid is at most kLptGridBytes, else the tile order.
  std::vector<int32_t> task_order;
  std::vector<int32_t> tile_tasks;  // ntiles + 1 offsets into tasks
  int win_rows = 0, win_cols = 0;   // largest window: (H + JBv - 1) x (W + JBu - 1)
  // Row stride of the windows in shared memory (the widest window); a batch's
  // lane l preferably holds an item whose window offset (win_offset) is l
  // mod 16.
  int win_stride = 0;
  // Group code of the items (PlanRequest::group); the register block of an
  // item is J + group_u - 1 cells wide and J + group_v - 1 high.
  int group = 1;
  // statistics
  int64_t occupied_cells = 0;
  int64_t real_items = 0;
  int max_cell_count = 0;
};

// Cells of a group along u and v (group code of PlanRequest::group).
PG_HD constexpr int group_u(int group) { return group == 1 ? 1 : 2; }
PG_HD constexpr int group_v(int group) { return group == 2 ? 2 : 1; }

// Offset of window cell (r, c) in a shared-memory window of row stride WS.
// Items of 2 x 2 groups sit at even rows and columns, which would leave
// their offsets r WS + c on even cells only (8 of the 16 bank pairs); one
// extra cell per two rows spreads them over all 16 while keeping the offset
// of (r + jv, c + ju) from (r, c) independent of r for even r.
PG_HD inline int win_offset(int r, int c, int WS, int group) {
  return r * WS + c + (group == 2 ? (r >> 1) : 0);
}
// Cells of a window of `rows` rows at row stride WS in that layout.
PG_HD inline int win_cells(int rows, int WS, int group) {
  return rows * WS + (group == 2 ? (rows + 1) / 2 : 0);
}

// Builds the plan.  Throws std::invalid_argument on bad input.
Plan build_plan(const PlanRequest &req);

// The column-walk plan of G^H (see walk_grid_kernel).  Tiles are those of the
// item plan (PlanRequest::tile <= 32), one task per occupied tile.  A warp's
// 32 lanes are the tile's rows; it walks the tile's base-cell columns in
// order, and at column q lane r takes the visibilities whose base cell is
// (r, q).  Slots follow that walk: per task, per column, per k = 0, 1, ...,
// the k-th visibility of every row that has more than k in that column, in
// row order.  There are no null slots (S = M): lane r's slot at step k is the
// column's running base plus the number of lower rows still active.
struct WalkPlan {
  int64_t M = 0;
  int T = 32;  // lanes (rows) per task block, and the column stride of counts
  std::vector<Task> tasks;          // one per occupied tile, in tile order
  std::vector<int32_t> task_order;  // launch order: most column steps first
  std::vector<int32_t> tile_tasks;  // ntiles + 1 offsets into tasks
  std::vector<int32_t> counts;      // tasks x T columns x 32 rows
  std::vector<int32_t> colstart;    // tasks x (T + 1): first slot of each column, then the end
  std::vector<double> frac_u, frac_v;  // per slot, as in Plan (t in [0, 1))
  std::vector<uint8_t> flip;
  std::vector<int32_t> slot_user;   // caller index of each slot
  int win_rows = 0, win_cols = 0;
  int win_stride = 0;   // odd, so that a column of 32 rows covers 16 bank pairs per half-warp
  int64_t steps = 0;    // sum over tasks and columns of the column's largest count
  int max_count = 0;    // largest count of one cell
  // Most steps of one warp: the sum of its columns' largest counts, with a
  // task's columns split over kWalkWarps warps as the kernel splits them.
  int max_warp_steps = 0;
};

// Builds the column-walk plan (group 1 only; every tile at most 32 x 32).
// Throws std::invalid_argument on bad input.
WalkPlan build_walk_plan(const PlanRequest &req);

// Splits [0, n) into ceil(n / tile) nearly equal ranges (>= 1 range).
AxisTiling make_tiling(int n, int tile);

}  // namespace pg
