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
}  // namespace

Plan build_plan(const PlanRequest &rq) {
  if (rq.M < 0) throw std::invalid_argument("negative number of visibilities");
  if (rq.M > 0 && (!rq.u || !rq.v)) throw std::invalid_argument("u and v must be given");
  if (rq.Ju < 1 || rq.Jv < 1) throw std::invalid_argument("kernel support must be >= 1");
  if (rq.Nu < 1 || rq.Nv < 1) throw std::invalid_argument("empty grid");
  if (rq.M > int64_t(INT32_MAX) - 1024)
    throw std::invalid_argument("more visibilities than int32 indices can address");
  if (rq.max_per_item < 1 || rq.max_per_item > 0xffff)
    throw std::invalid_argument("max_per_item out of range");

  Plan P;
  P.M = rq.M;
  P.Nu = rq.Nu;
  P.Nv = rq.Nv;
  P.Ju = rq.Ju;
  P.Jv = rq.Jv;
  P.tu = make_tiling(rq.Nu, rq.tile);
  P.tv = make_tiling(rq.Nv, rq.tile);
  // A window reaches J - 1 cells into the next tile; it must not reach two
  // tiles ahead, so every tile must be at least J - 1 cells wide.
  const int min_w = P.tu.start[1] - P.tu.start[0];
  const int min_h = P.tv.start[1] - P.tv.start[0];
  for (int b = 0; b < P.tu.n; ++b)
    if (P.tu.start[b + 1] - P.tu.start[b] < rq.Ju - 1 || rq.Nu < rq.Ju)
      throw std::invalid_argument("grid width is smaller than the kernel support");
  for (int b = 0; b < P.tv.n; ++b)
    if (P.tv.start[b + 1] - P.tv.start[b] < rq.Jv - 1 || rq.Nv < rq.Jv)
      throw std::invalid_argument("grid height is smaller than the kernel support");
  (void)min_w;
  (void)min_h;

  const int ntu = P.tu.n, ntv = P.tv.n, ntiles = ntu * ntv;
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
#pragma omp parallel for schedule(static)
  for (int64_t m = 0; m < M; ++m) {
    const double su = rq.u[m] - rq.Ju * 0.5, sv = rq.v[m] - rq.Jv * 0.5;
    const double ku = std::floor(su), kv = std::floor(sv);
    tu[m] = su - ku;
    tv[m] = sv - kv;
    const int q0 = int(wrap(ku + 1, rq.Nu));
    const int p0 = int(wrap(kv + 1, rq.Nv));
    // exp(-2 pi i ((k_u + j_u) + (k_v + j_v)) / 2) = (-1)^(k_u + k_v) (-1)^(j_u + j_v);
    // the first factor goes into the weight, the second into the polynomials.
    flip[m] = uint8_t((int64_t(ku) + int64_t(kv)) & 1);
    const int a = P.tv.of[p0], b = P.tu.of[q0];
    const int t = a * ntu + b;
    const int w = P.tu.start[b + 1] - P.tu.start[b];
    rank[m] = tile_cell0[t] + int64_t(p0 - P.tv.start[a]) * w + (q0 - P.tu.start[b]);
  }

  // Stable counting sort by cell rank.
  std::vector<int64_t> cell_first(ncells + 1, 0);
  for (int64_t m = 0; m < M; ++m) cell_first[rank[m] + 1]++;
  for (int64_t c = 0; c < ncells; ++c) cell_first[c + 1] += cell_first[c];
  P.perm.resize(M);
  {
    std::vector<int64_t> fill(cell_first.begin(), cell_first.end() - 1);
    for (int64_t m = 0; m < M; ++m) P.perm[fill[rank[m]]++] = int32_t(m);
  }
  P.frac_u.resize(M);
  P.frac_v.resize(M);
  P.weight.resize(M);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i) {
    const int32_t m = P.perm[i];
    P.frac_u[i] = tu[m];
    P.frac_v[i] = tv[m];
    std::complex<double> wgt = rq.weights ? rq.weights[m] : std::complex<double>(1.0, 0.0);
    P.weight[i] = flip[m] ? -wgt : wgt;
  }

  // Work items, tile by tile.  A cell with c visibilities becomes
  // ceil(c / K) items of nearly equal size.  Items are grouped in layers by
  // chunk index, so a layer never holds two items of one cell; each layer is
  // ordered by descending size (lanes of a batch then run equal loops) and
  // padded to a whole number of 32-item batches.  Any batch therefore holds
  // at most one item per base cell.
  const int K = rq.max_per_item;
  P.tile_tasks.assign(ntiles + 1, 0);
  struct Item {
    int32_t first, lp, lq, count, chunk;
  };
  std::vector<Item> items;
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
        const int lp = local / w, lq = local % w;
        const int64_t chunks = (n + K - 1) / K;
        const int64_t base = n / chunks, rem = n % chunks;
        int64_t first = cell_first[c];
        for (int64_t k = 0; k < chunks; ++k) {
          const int32_t cnt = int32_t(base + (k < rem ? 1 : 0));
          items.push_back({int32_t(first), lp, lq, cnt, int32_t(k)});
          first += cnt;
        }
      }
      P.real_items += int64_t(items.size());
      const int64_t item0 = int64_t(P.item_first.size());
      // Layer order: chunk index ascending, then size descending; stable, so
      // items of equal size keep their cell order.
      std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) {
        return x.chunk != y.chunk ? x.chunk < y.chunk : x.count > y.count;
      });
      for (size_t k = 0; k < items.size(); ++k) {
        if (k > 0 && items[k].chunk != items[k - 1].chunk)
          while ((P.item_first.size() - item0) % kBatch) {
            P.item_first.push_back(0);
            P.item_code.push_back(0);
          }
        P.item_first.push_back(items[k].first);
        P.item_code.push_back(item_pack(items[k].lp, items[k].lq, items[k].count));
      }
      while ((P.item_first.size() - item0) % kBatch) {
        P.item_first.push_back(0);
        P.item_code.push_back(0);
      }
      const int64_t nb = (int64_t(P.item_first.size()) - item0) / kBatch;
      const int64_t b0 = item0 / kBatch;
      for (int64_t s = 0; s < nb; s += rq.max_batches_per_task) {
        Task tk{};
        tk.P = P.tv.start[a];
        tk.Q = P.tu.start[b];
        tk.H = h;
        tk.W = w;
        tk.batch_begin = int32_t(b0 + s);
        tk.batch_end = int32_t(b0 + std::min<int64_t>(nb, s + rq.max_batches_per_task));
        tk.tile = t;
        P.tasks.push_back(tk);
      }
      P.tile_tasks[t + 1] = int32_t(P.tasks.size());
      P.win_rows = std::max(P.win_rows, h + rq.Jv - 1);
      P.win_cols = std::max(P.win_cols, w + rq.Ju - 1);
    }
  if (P.item_first.size() > size_t(INT32_MAX))
    throw std::invalid_argument("too many work items for int32 indexing");
  return P;
}

}  // namespace pg
