// Coverage planning (host, FP64): everything about a set of visibilities that
// does not change between applies of the operator.
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
  int max_per_item = 16;        // visibilities of one cell handled by one lane
  int max_batches_per_task = 64;
};

// Tiling of one grid axis: tile b covers [start[b], start[b + 1]).
struct AxisTiling {
  int n = 0;
  std::vector<int32_t> start;  // n + 1 entries
  std::vector<int32_t> of;     // axis length entries: tile index of each cell
};

struct Plan {
  int64_t M = 0;
  int Nu = 0, Nv = 0, Ju = 0, Jv = 0;
  AxisTiling tu, tv;                 // tilings of the u (columns) and v (rows) axes
  std::vector<double> frac_u, frac_v;  // plan order, in [0, 1)
  std::vector<std::complex<double>> weight;  // plan order, phase sign folded in
  std::vector<int32_t> perm;         // plan order -> caller order
  std::vector<int32_t> item_first;   // per work item
  std::vector<int32_t> item_code;    // per work item (item_pack)
  std::vector<Task> tasks;
  std::vector<int32_t> tile_tasks;   // ntiles + 1 offsets into tasks
  int win_rows = 0, win_cols = 0;    // largest window: (H + Jv - 1) x (W + Ju - 1)
  // statistics
  int64_t occupied_cells = 0;
  int64_t real_items = 0;
  int max_cell_count = 0;
};

// Builds the plan.  Throws std::invalid_argument on bad input.
Plan build_plan(const PlanRequest &req);

// Splits [0, n) into ceil(n / tile) nearly equal ranges (>= 1 range).
AxisTiling make_tiling(int n, int tile);

}  // namespace pg
