#include "plan.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <string>

namespace pg {

AxisTiling make_tiling(int n, int tile) {
  AxisTiling t;
  t.n = std::max(1, (n + tile - 1) / tile);
  t.start.resize(t.n + 1);
  for (int b = 0; b <= t.n; ++b) t.start[b] = int32_t(int64_t(b) * n / t.n);
  t.of.resize(n);
  for (int b = 0; b < t.n; ++b)
    for (int c = t.start[b]; c < t.start[b + 1]; ++c) t.of[c] = b;
  return t;
}

namespace {
// utilities::mod (cpp/purify/utilities.cc:350-357): fmod wrapped to [0, y).
double wrap(double x, double y) {
  double r = std::fmod(x, y);
  if (r < 0) r += y;
  return r;
}

// Most items of one shared-memory bank class in a batch (see the packing).
// At the 10^7-visibility workload a lane-block access then costs about 3.2
// shared-memory wavefronts instead of 5.0 (2 is the floor) for 2% more
// slots; a cap of 3 over the whole batch cost 3.4% slots and measured
// slower, a cap of 2 cost 16%.
constexpr int kClassCap = 4;

struct Item {
  int32_t first;  // first visibility in cell-sorted order
  int32_t count;
  int32_t cell;   // cell index inside the tile
  int32_t lp, lq;
};

// Batch order inside each task for the kernels' round-robin dealing (batch
// i of a task goes to warp i mod nw).  A batch costs about kStepCost per
// k-step plus kFlushCost for its block flush (warp instructions of the grid
// kernel at J = 6).  The batches are taken heaviest first in rounds of nw;
// in each round the heaviest goes to the warp with the least work so far.
// The last, partial round goes to the lightest warps, and the warps are then
// numbered by load so that round-robin dealing gives every warp its list.
// On the 10^7-visibility workload this takes the mean over tasks of (mean
// warp load / largest warp load) from 0.86 (plain longest-first order) to
// 0.96.  Only the order of the batch records changes; slots stay put.
constexpr int64_t kStepCost = 220, kFlushCost = 180;

void balance_task_batches(Plan &P, int nw) {
  if (nw <= 1) return;
  std::vector<int32_t> order, wl(nw), pos;
  std::vector<int64_t> load(nw);
  std::vector<std::vector<int32_t>> lists(nw);
  std::vector<int32_t> base, kmax, code;
  for (const Task &tk : P.tasks) {
    const int b0 = tk.batch_begin, n = tk.batch_end - tk.batch_begin;
    if (n <= 1) continue;
    auto cost = [&](int i) { return kStepCost * P.batch_kmax[b0 + i] + kFlushCost; };
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
    std::fill(load.begin(), load.end(), 0);
    for (auto &l : lists) l.clear();
    const int full = n / nw, rem = n - full * nw;
    auto by_load = [&] {
      std::iota(wl.begin(), wl.end(), 0);
      std::stable_sort(wl.begin(), wl.end(), [&](int x, int y) { return load[x] < load[y]; });
    };
    for (int r = 0; r < full; ++r) {
      by_load();
      for (int j = 0; j < nw; ++j) {
        const int b = order[size_t(r) * nw + j];
        lists[wl[j]].push_back(b);
        load[wl[j]] += cost(b);
      }
    }
    by_load();
    for (int j = 0; j < rem; ++j) lists[wl[j]].push_back(order[size_t(full) * nw + j]);
    // warp label j runs lists[wl[j]]: its r-th batch goes to position r nw + j
    pos.assign(n, -1);
    for (int j = 0; j < nw; ++j)
      for (size_t r = 0; r < lists[wl[j]].size(); ++r) pos[r * nw + j] = lists[wl[j]][r];
    base.assign(P.batch_base.begin() + b0, P.batch_base.begin() + b0 + n);
    kmax.assign(P.batch_kmax.begin() + b0, P.batch_kmax.begin() + b0 + n);
    code.assign(P.lane_code.begin() + size_t(b0) * kBatch,
                P.lane_code.begin() + size_t(b0 + n) * kBatch);
    for (int i = 0; i < n; ++i) {
      const int src = pos[i];
      if (src < 0) throw std::logic_error("balance_task_batches: unfilled position");
      P.batch_base[b0 + i] = base[src];
      P.batch_kmax[b0 + i] = kmax[src];
      std::copy(code.begin() + size_t(src) * kBatch, code.begin() + size_t(src + 1) * kBatch,
                P.lane_code.begin() + size_t(b0 + i) * kBatch);
    }
  }
}
}  // namespace

Plan build_plan(const PlanRequest &rq) {
  if (rq.M < 0) throw std::invalid_argument("negative number of visibilities");
  if (rq.M > 0 && (!rq.u || !rq.v)) throw std::invalid_argument("u and v must be given");
  if (rq.Ju < 1 || rq.Jv < 1) throw std::invalid_argument("kernel support must be >= 1");
  if (rq.Nu < 1 || rq.Nv < 1) throw std::invalid_argument("empty grid");
  if (rq.M > int64_t(INT32_MAX) / 2)
    throw std::invalid_argument("more visibilities than int32 slot indices can address");
  if (rq.max_per_item < 1 || rq.max_per_item > 0xffff)
    throw std::invalid_argument("max_per_item out of range");
  if (rq.tile < 1 || rq.tile > 255) throw std::invalid_argument("tile edge out of range");
  if (rq.max_batches_per_task < 1 || rq.max_batches_per_task > kMaxTaskBatches)
    throw std::invalid_argument("max_batches_per_task out of range");
  if (rq.group < 1 || rq.group > 3) throw std::invalid_argument("group must be 1, 2 or 3");
  if (rq.class_cap < 0 || rq.class_cap > 16) throw std::invalid_argument("class_cap out of range");
  for (int64_t m = 0; m < rq.M; ++m)
    if (!std::isfinite(rq.u[m]) || !std::isfinite(rq.v[m]))
      throw std::invalid_argument("visibility " + std::to_string(m) +
                                  " has a non-finite u or v coordinate");

  Plan P;
  P.M = rq.M;
  P.Nu = rq.Nu;
  P.Nv = rq.Nv;
  P.Ju = rq.Ju;
  P.Jv = rq.Jv;
  P.group = rq.group;
  const int G = rq.group, GU = group_u(G), GV = group_v(G);
  const int class_cap = rq.class_cap > 0 ? rq.class_cap : kClassCap;
  // register block of an item: the support plus the extra cell of a group
  const int JBu = rq.Ju + GU - 1, JBv = rq.Jv + GV - 1;
  P.tu = make_tiling(rq.Nu, rq.tile);
  P.tv = make_tiling(rq.Nv, rq.tile);
  // A window reaches JB - 1 cells into the next tile; it must not reach two
  // tiles ahead, so every tile must be at least JB - 1 cells wide, and the
  // grid must hold the support.
  if (rq.Nu < rq.Ju || rq.Nv < rq.Jv)
    throw std::invalid_argument("grid is smaller than the kernel support");
  for (int b = 0; b < P.tu.n; ++b)
    if (P.tu.start[b + 1] - P.tu.start[b] < JBu - 1)
      throw std::invalid_argument("grid width is too small for the kernel support");
  for (int b = 0; b < P.tv.n; ++b)
    if (P.tv.start[b + 1] - P.tv.start[b] < JBv - 1)
      throw std::invalid_argument("grid height is too small for the kernel support");

  const int ntu = P.tu.n, ntv = P.tv.n, ntiles = ntu * ntv;
  // Row stride of the tasks' shared-memory windows: the widest window.
  int WS = 0;
  for (int b = 0; b < ntu; ++b) WS = std::max(WS, P.tu.start[b + 1] - P.tu.start[b] + JBu - 1);
  // Row pairs anchor at even columns: an odd stride keeps their offsets on
  // all 16 bank pairs.
  if (G == 3) WS |= 1;
  P.win_stride = WS;
  // Cell rank: tiles in row-major order, cells row-major inside a tile.
  std::vector<int64_t> tile_cell0(ntiles + 1, 0);
  for (int a = 0; a < ntv; ++a)
    for (int b = 0; b < ntu; ++b) {
      const int t = a * ntu + b;
      const int64_t h = P.tv.start[a + 1] - P.tv.start[a];
      const int64_t w = P.tu.start[b + 1] - P.tu.start[b];
      tile_cell0[t + 1] = tile_cell0[t] + h * w;
    }
  const int64_t ncells = tile_cell0[ntiles];

  // Per-visibility coordinates in FP64 (operators.cc:34-41): k = floor(u - J/2)
  // is the cell before the first tap, taps sit at k + 1 .. k + J (mod N), and
  // the kernel is evaluated at u - (k + j) = t + J/2 - j with t = u - J/2 - k.
  const int64_t M = rq.M;
  std::vector<double> tu(M), tv(M);
  std::vector<int64_t> rank(M);
  std::vector<uint8_t> flip(M);
  // With groups, a visibility's base cell inside its group (dx, dy) is added
  // to its fractions and the item is keyed by the group's anchor cell.
  const int umask = ~(GU - 1), vmask = ~(GV - 1);
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < M; ++m) {
    const double su = rq.u[m] - rq.Ju * 0.5, sv = rq.v[m] - rq.Jv * 0.5;
    const double ku = std::floor(su), kv = std::floor(sv);
    tu[m] = su - ku;
    tv[m] = sv - kv;
    const int q0 = int(wrap(ku + 1, rq.Nu));
    const int p0 = int(wrap(kv + 1, rq.Nv));
    // exp(-2 pi i ((k_u + j_u) + (k_v + j_v)) / 2) = (-1)^(k_u + k_v) (-1)^(j_u + j_v);
    // the first factor goes with the weight, the second into the polynomials.
    flip[m] = uint8_t((int64_t(ku) + int64_t(kv)) & 1);
    const int a = P.tv.of[p0], b = P.tu.of[q0];
    const int t = a * ntu + b;
    const int w = P.tu.start[b + 1] - P.tu.start[b];
    const int lp = p0 - P.tv.start[a], lq = q0 - P.tu.start[b];
    const int ap = lp & vmask, aq = lq & umask;
    tu[m] += double(lq - aq);
    tv[m] += double(lp - ap);
    rank[m] = tile_cell0[t] + int64_t(ap) * w + aq;
  }
  if (rq.weights)
    for (int64_t m = 0; m < M && P.unit_weights; ++m)
      if (rq.weights[m] != std::complex<double>(1.0, 0.0)) P.unit_weights = false;

  // Stable counting sort by cell rank: sorted[k] is a caller index.
  std::vector<int64_t> cell_first(ncells + 1, 0);
  for (int64_t m = 0; m < M; ++m) cell_first[rank[m] + 1]++;
  for (int64_t c = 0; c < ncells; ++c) cell_first[c + 1] += cell_first[c];
  std::vector<int32_t> sorted(M);
  {
    std::vector<int64_t> fill(cell_first.begin(), cell_first.end() - 1);
    for (int64_t m = 0; m < M; ++m) sorted[fill[rank[m]]++] = int32_t(m);
  }

  // Work items and batches, tile by tile.
  const int K = rq.max_per_item;
  P.tile_tasks.assign(ntiles + 1, 0);
  std::vector<Item> items;
  std::vector<int32_t> stamp;  // per cell of the tile: last batch that took it
  std::vector<uint8_t> taken;
  // slot assignment collected per batch: (slot, sorted index) pairs
  std::vector<int64_t> slot_sorted;  // slot -> sorted index or -1
  for (int a = 0; a < ntv; ++a)
    for (int b = 0; b < ntu; ++b) {
      const int t = a * ntu + b;
      const int h = P.tv.start[a + 1] - P.tv.start[a];
      const int w = P.tu.start[b + 1] - P.tu.start[b];
      items.clear();
      for (int64_t c = tile_cell0[t]; c < tile_cell0[t + 1]; ++c) {
        const int64_t n = cell_first[c + 1] - cell_first[c];
        if (n == 0) continue;
        P.occupied_cells++;
        P.max_cell_count = std::max<int64_t>(P.max_cell_count, n);
        const int local = int(c - tile_cell0[t]);
        const int64_t chunks = (n + K - 1) / K;
        const int64_t base = n / chunks, rem = n % chunks;
        int64_t first = cell_first[c];
        for (int64_t k = 0; k < chunks; ++k) {
          const int32_t cnt = int32_t(base + (k < rem ? 1 : 0));
          items.push_back({int32_t(first), cnt, local, local / w, local % w});
          first += cnt;
        }
      }
      P.real_items += int64_t(items.size());
      // Longest items first (lanes of a batch then run equal loops); stable,
      // so equal sizes keep cell order.
      std::stable_sort(items.begin(), items.end(),
                       [](const Item &x, const Item &y) { return x.count > y.count; });
      // Greedy packing: scan the pending items in order and take one unless
      // its base cell is already in the batch or the batch already holds
      // too many items of its bank class; a scan gives up 256 clashes past
      // the first pending item.  The first scan takes only items of the front
      // item's count, at most two per class; the second fills the batch from
      // the front at kClassCap per class.  The bank class of an item is its window
      // offset lp * WS + lq mod 16: at every (jv, ju) offset of their blocks,
      // the lanes of a half-warp that share a class hit the same 8-byte bank
      // pair, and each extra one costs a shared-memory wavefront.  An item of
      // class r goes to lane r or 16 + r when free, else to a free lane of
      // the half-warp holding fewer items of class r; with the cap, a
      // half-warp then holds at most two items of a class.
      stamp.assign(size_t(h) * w, -1);
      taken.assign(items.size(), 0);
      size_t front = 0;
      int32_t batch_id = 0;
      const int64_t task_batch0 = int64_t(P.batch_base.size());
      std::vector<int64_t> lane_item(kBatch);
      while (true) {
        while (front < items.size() && taken[front]) ++front;
        if (front == items.size()) break;
        std::fill(lane_item.begin(), lane_item.end(), -1);
        int class_count[16] = {0};
        int half_class[2][16] = {{0}};
        int filled = 0;
        // one scan from the front: cap items per class; with same_count >= 0
        // only the items of that count (a contiguous run of the sorted list)
        auto scan = [&](int cap, int same_count) {
          size_t skipped = 0;
          for (size_t k = front; k < items.size() && filled < kBatch; ++k) {
            if (same_count >= 0 && items[k].count != same_count) break;
            if (taken[k]) continue;
            const int r = win_offset(items[k].lp, items[k].lq, WS, G) & 15;
            int lane = lane_item[r] < 0 ? r : (lane_item[16 + r] < 0 ? 16 + r : -1);
            if (lane < 0) {
              // both class lanes taken: a free lane in the half-warp holding
              // fewer items of this class
              const int h0 = half_class[0][r] <= half_class[1][r] ? 0 : 1;
              for (int hh = 0; hh < 2 && lane < 0; ++hh) {
                const int h = hh == 0 ? h0 : 1 - h0;
                for (int l = 16 * h; l < 16 * h + 16; ++l)
                  if (lane_item[l] < 0) {
                    lane = l;
                    break;
                  }
              }
            }
            if (stamp[items[k].cell] == batch_id || lane < 0 || class_count[r] >= cap) {
              if (++skipped > 256) break;
              continue;
            }
            ++class_count[r];
            ++half_class[lane >> 4][r];
            stamp[items[k].cell] = batch_id;
            taken[k] = 1;
            lane_item[lane] = int64_t(k);
            ++filled;
          }
        };
        // first the items of the front item's count (no null slots among
        // them) at two per class, then the rest of the batch at kClassCap
        scan(std::min(2, class_cap), items[front].count);
        scan(class_cap, -1);
        int kmax = 0;
        for (int l = 0; l < kBatch; ++l)
          if (lane_item[l] >= 0) kmax = std::max(kmax, int(items[lane_item[l]].count));
        const int64_t base = P.S;
        P.batch_base.push_back(int32_t(base));
        P.batch_kmax.push_back(kmax);
        P.S += int64_t(kBatch) * kmax;
        if (P.S > int64_t(INT32_MAX)) throw std::invalid_argument("too many slots");
        slot_sorted.resize(P.S, -1);
        for (int l = 0; l < kBatch; ++l) {
          if (lane_item[l] >= 0) {
            const Item &it = items[lane_item[l]];
            P.lane_code.push_back(item_pack(it.lp, it.lq, it.count));
            for (int k = 0; k < it.count; ++k)
              slot_sorted[base + int64_t(kBatch) * k + l] = it.first + k;
          } else {
            P.lane_code.push_back(0);
          }
        }
        ++batch_id;
      }
      // Tasks: consecutive batches of the tile, bounded in slots and batches.
      const int64_t nb = int64_t(P.batch_base.size()) - task_batch0;
      int64_t s = 0;
      while (s < nb) {
        int64_t e = s, slots = 0;
        while (e < nb && (e == s || (e - s < rq.max_batches_per_task &&
                                     slots + int64_t(kBatch) * P.batch_kmax[task_batch0 + e] <=
                                         rq.max_slots_per_task))) {
          slots += int64_t(kBatch) * P.batch_kmax[task_batch0 + e];
          ++e;
        }
        Task tk{};
        tk.P = P.tv.start[a];
        tk.Q = P.tu.start[b];
        tk.H = h;
        tk.W = w;
        tk.batch_begin = int32_t(task_batch0 + s);
        tk.batch_end = int32_t(task_batch0 + e);
        tk.tile = t;
        P.tasks.push_back(tk);
        s = e;
      }
      P.tile_tasks[t + 1] = int32_t(P.tasks.size());
      P.win_rows = std::max(P.win_rows, h + JBv - 1);
      P.win_cols = std::max(P.win_cols, w + JBu - 1);
    }

  // Windows are sized and strided by win_cols: with row pairs the stride is
  // the odd WS, which may be one wider than the widest window.
  P.win_cols = std::max(P.win_cols, WS);
  balance_task_batches(P, rq.warps);

  // Launch order.  Longest tasks first makes the last wave of CTAs short;
  // that pays while the grid stays in L2 (<= kLptGridBytes as complex<float>).
  // A larger grid keeps the spatial (tile) order, which reuses the halos of
  // neighbouring windows from L2.
  P.task_order.resize(P.tasks.size());
  std::iota(P.task_order.begin(), P.task_order.end(), 0);
  if (int64_t(rq.Nu) * rq.Nv * 8 <= kLptGridBytes) {
    std::vector<int64_t> cost(P.tasks.size(), 0);
    for (size_t k = 0; k < P.tasks.size(); ++k)
      for (int b = P.tasks[k].batch_begin; b < P.tasks[k].batch_end; ++b) cost[k] += P.batch_kmax[b];
    std::stable_sort(P.task_order.begin(), P.task_order.end(),
                     [&](int32_t x, int32_t y) { return cost[x] > cost[y]; });
  }
  // Per-slot coverage state.
  const int64_t S = P.S;
  P.frac_u.assign(S, 0.0);
  P.frac_v.assign(S, 0.0);
  P.flip.assign(S, 0);
  P.slot_user.assign(S, -1);
  P.user_slot.assign(M, -1);
  if (!P.unit_weights) P.weight.assign(S, std::complex<double>(0.0, 0.0));
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < S; ++s) {
    const int64_t k = slot_sorted[s];
    if (k < 0) continue;
    const int32_t m = sorted[k];
    P.frac_u[s] = tu[m];
    P.frac_v[s] = tv[m];
    P.flip[s] = flip[m];
    P.slot_user[s] = m;
    P.user_slot[m] = int32_t(s);
    if (!P.unit_weights) {
      const std::complex<double> wgt = rq.weights[m];
      P.weight[s] = flip[m] ? -wgt : wgt;
    }
  }
  return P;
}

WalkPlan build_walk_plan(const PlanRequest &rq) {
  if (rq.M < 0 || (rq.M > 0 && (!rq.u || !rq.v)))
    throw std::invalid_argument("bad visibility coordinates");
  if (rq.group != 1) throw std::invalid_argument("the column walk takes single-cell items only");
  if (rq.Ju < 1 || rq.Jv < 1 || rq.Nu < rq.Ju || rq.Nv < rq.Jv)
    throw std::invalid_argument("kernel support and grid do not fit");
  if (rq.M > int64_t(INT32_MAX) / 2)
    throw std::invalid_argument("more visibilities than int32 slot indices can address");
  WalkPlan W;
  W.M = rq.M;
  const AxisTiling tu = make_tiling(rq.Nu, rq.tile), tv = make_tiling(rq.Nv, rq.tile);
  const int ntu = tu.n, ntv = tv.n, ntiles = ntu * ntv, T = W.T;
  int wmax = 0, hmax = 0;
  for (int b = 0; b < ntu; ++b) wmax = std::max(wmax, tu.start[b + 1] - tu.start[b]);
  for (int a = 0; a < ntv; ++a) hmax = std::max(hmax, tv.start[a + 1] - tv.start[a]);
  if (wmax > T || hmax > T) throw std::invalid_argument("the column walk needs tiles of at most 32");
  for (int b = 0; b < ntu; ++b)
    if (tu.start[b + 1] - tu.start[b] < rq.Ju - 1)
      throw std::invalid_argument("grid width is too small for the kernel support");
  for (int a = 0; a < ntv; ++a)
    if (tv.start[a + 1] - tv.start[a] < rq.Jv - 1)
      throw std::invalid_argument("grid height is too small for the kernel support");
  W.win_rows = hmax + rq.Jv - 1;
  W.win_cols = wmax + rq.Ju - 1;
  W.win_stride = W.win_cols | 1;

  // Per visibility, as build_plan with group 1: fractions, phase flip, tile
  // and the base cell (row lp, column lq) inside it.
  const int64_t M = rq.M;
  std::vector<double> fu(M), fv(M);
  std::vector<uint8_t> flip(M);
  std::vector<int32_t> tile(M);
  std::vector<int16_t> row(M), col(M);
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < M; ++m) {
    const double su = rq.u[m] - rq.Ju * 0.5, sv = rq.v[m] - rq.Jv * 0.5;
    const double ku = std::floor(su), kv = std::floor(sv);
    fu[m] = su - ku;
    fv[m] = sv - kv;
    const int q0 = int(wrap(ku + 1, rq.Nu));
    const int p0 = int(wrap(kv + 1, rq.Nv));
    flip[m] = uint8_t((int64_t(ku) + int64_t(kv)) & 1);
    const int a = tv.of[p0], b = tu.of[q0];
    tile[m] = a * ntu + b;
    row[m] = int16_t(p0 - tv.start[a]);
    col[m] = int16_t(q0 - tu.start[b]);
  }
  // Cells: tile-major, then column, then row; visibilities of a cell in
  // caller order (stable counting sort).
  const int64_t cells = int64_t(ntiles) * T * T;
  std::vector<int64_t> cell_first(cells + 1, 0);
  auto cell_of = [&](int64_t m) { return (int64_t(tile[m]) * T + col[m]) * T + row[m]; };
  for (int64_t m = 0; m < M; ++m) cell_first[cell_of(m) + 1]++;
  for (int64_t c = 0; c < cells; ++c) cell_first[c + 1] += cell_first[c];
  std::vector<int32_t> sorted(M);
  {
    std::vector<int64_t> fill(cell_first.begin(), cell_first.end() - 1);
    for (int64_t m = 0; m < M; ++m) sorted[fill[cell_of(m)]++] = int32_t(m);
  }
  // Tasks: occupied tiles in tile order.
  W.tile_tasks.assign(ntiles + 1, 0);
  std::vector<int32_t> task_tile;
  for (int t = 0; t < ntiles; ++t) {
    if (cell_first[int64_t(t + 1) * T * T] > cell_first[int64_t(t) * T * T]) {
      const int a = t / ntu, b = t % ntu;
      Task tk{};
      tk.P = tv.start[a];
      tk.Q = tu.start[b];
      tk.H = tv.start[a + 1] - tv.start[a];
      tk.W = tu.start[b + 1] - tu.start[b];
      tk.tile = t;
      W.tasks.push_back(tk);
      task_tile.push_back(t);
    }
    W.tile_tasks[t + 1] = int32_t(W.tasks.size());
  }
  const int64_t ntasks = int64_t(W.tasks.size());
  W.counts.assign(size_t(ntasks) * T * T, 0);
  W.colstart.assign(size_t(ntasks) * (T + 1), 0);
  std::vector<int64_t> cost(ntasks, 0);
  // Slot positions: the walk order within each task; task k's slots start
  // at the number of visibilities of the tasks before it.
  std::vector<int32_t> slot_of_sorted(M);
  int max_count = 0, max_warp_steps = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(max : max_count, max_warp_steps)
  for (int64_t k = 0; k < ntasks; ++k) {
    const int64_t c0 = int64_t(task_tile[k]) * T * T;
    const int wk = W.tasks[k].W;
    int64_t s = cell_first[c0];  // visibilities before this tile, in tile order
    int warp_steps[kWalkWarps] = {0};
    for (int q = 0; q < T; ++q) {
      W.colstart[size_t(k) * (T + 1) + q] = int32_t(s);
      int kmax = 0;
      for (int r = 0; r < T; ++r) {
        const int n = int(cell_first[c0 + int64_t(q) * T + r + 1] - cell_first[c0 + int64_t(q) * T + r]);
        W.counts[(size_t(k) * T + q) * T + r] = n;
        kmax = std::max(kmax, n);
      }
      max_count = std::max(max_count, kmax);
      cost[k] += kmax;
      for (int w = 0; w < kWalkWarps; ++w)
        if (q >= w * wk / kWalkWarps && q < (w + 1) * wk / kWalkWarps) warp_steps[w] += kmax;
      for (int j = 0; j < kmax; ++j)
        for (int r = 0; r < T; ++r) {
          const int64_t c = c0 + int64_t(q) * T + r;
          if (cell_first[c + 1] - cell_first[c] > j) slot_of_sorted[cell_first[c] + j] = int32_t(s++);
        }
    }
    W.colstart[size_t(k) * (T + 1) + T] = int32_t(s);
    for (int w = 0; w < kWalkWarps; ++w) max_warp_steps = std::max(max_warp_steps, warp_steps[w]);
  }
  W.max_count = max_count;
  W.max_warp_steps = max_warp_steps;
  for (int64_t k = 0; k < ntasks; ++k) W.steps += cost[k];
  W.task_order.resize(ntasks);
  std::iota(W.task_order.begin(), W.task_order.end(), 0);
  std::stable_sort(W.task_order.begin(), W.task_order.end(),
                   [&](int32_t x, int32_t y) { return cost[x] > cost[y]; });
  W.frac_u.assign(M, 0.0);
  W.frac_v.assign(M, 0.0);
  W.flip.assign(M, 0);
  W.slot_user.assign(M, -1);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i) {
    const int32_t m = sorted[i];
    const int64_t s = slot_of_sorted[i];
    W.frac_u[s] = fu[m];
    W.frac_v[s] = fv[m];
    W.flip[s] = flip[m];
    W.slot_user[s] = m;
  }
  return W;
}

}  // namespace pg
