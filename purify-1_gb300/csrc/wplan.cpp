#include "wplan.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <string>

#include "gridding_kernels.h"

namespace pg {
namespace {
constexpr double kPi = 3.14159265358979323846;

double wrap(double x, double y) {
  double r = std::fmod(x, y);
  if (r < 0) r += y;
  return r;
}

// projection_kernels::pixel_to_lambda (projection_kernels.cc:28-30)
double pixel_to_lambda(double cell, int imsize, double os) {
  return 60. * 60. * 180. / cell / std::floor(os * imsize) / kPi;
}

// The zero-padded linear convolution of convolution.h:42-52,
// out(j) = sum_k f(k) g_pad(n_out - 1 - j + k), n_out = Jg + Jf - 1.
void conv1d(const double *f, int Jf, const std::complex<double> *g, int Jg,
            std::complex<double> *out) {
  const int n_out = Jg + Jf - 1;
  for (int j = 0; j < n_out; ++j) {
    std::complex<double> acc = 0;
    for (int k = 0; k < Jf; ++k) {
      const int idx = n_out - 1 - j + k - (Jf - 1);  // index into the unpadded g
      if (idx >= 0 && idx < Jg) acc += f[k] * g[idx];
    }
    out[j] = acc;
  }
}

// Which of the three terms of a row's sample matrix
//   g = (a~ / (w i)) b~^T + (1 - chi_v) 1^T + chi_v (1 - chi_u)^T
// are nonzero (bit r for term r), from the validity masks chi of
// projection_kernels.cc:38-45 at the row's Jw sample offsets.  A term that is
// zero here is exactly zero, so leaving it out changes no tap.
int row_terms(double u, double v, double w, int Jw, double dul, double dvl) {
  const double dwu = u - std::floor(u - Jw * 0.5), dwv = v - std::floor(v - Jw * 0.5);
  bool any_u = false, all_u = true, any_v = false, all_v = true;
  for (int k = 0; k < Jw; ++k) {
    const double U = dwu - k - 1, V = dwv - k - 1;
    const bool ok_u = std::abs(U * dul / w) < 1, ok_v = std::abs(V * dvl / w) < 1;
    any_u |= ok_u;
    all_u &= ok_u;
    any_v |= ok_v;
    all_v &= ok_v;
  }
  return int(any_v && any_u) | int(!all_v) << 1 | int(any_v && !all_u) << 2;
}
}  // namespace

WPlan build_wplan(const WPlanRequest &rq) {
  if (rq.M < 0) throw std::invalid_argument("negative number of visibilities");
  if (rq.M > 0 && (!rq.u || !rq.v || (!rq.w && !rq.plain)))
    throw std::invalid_argument("u, v and w must be given");
  if (rq.J < 1 || rq.Jw < 1) throw std::invalid_argument("kernel supports must be >= 1");
  if (rq.plain && (rq.Ju < 1 || rq.Jv < 1)) throw std::invalid_argument("kernel supports must be >= 1");
  if (rq.M > int64_t(INT32_MAX) - 1) throw std::invalid_argument("too many visibilities");
  for (int64_t m = 0; m < rq.M; ++m)
    if (!std::isfinite(rq.u[m]) || !std::isfinite(rq.v[m]) || (!rq.plain && !std::isfinite(rq.w[m])))
      throw std::invalid_argument("visibility " + std::to_string(m) +
                                  " has a non-finite u, v or w coordinate");
  WPlan P;
  P.M = rq.M;
  P.Nu = rq.Nu;
  P.Nv = rq.Nv;
  P.plain = rq.plain;
  P.Ju = rq.Ju;
  P.Jv = rq.Jv;
  // plain rows: S = max(Ju, Jv) for every row (a w-support of 1 on a support
  // of S cells)
  const int Jrow = rq.plain ? std::max(rq.Ju, rq.Jv) : rq.J;
  P.J = Jrow;
  const int64_t M = rq.M;
  std::vector<int32_t> jw(M);
  int Smax = 1;
  for (int64_t m = 0; m < M; ++m) {
    jw[m] = rq.plain ? 1 : (rq.jw_rows ? rq.jw_rows[m] : rq.Jw);
    if (jw[m] < 1 || jw[m] + Jrow - 1 > 255) throw std::invalid_argument("w-support out of range");
    Smax = std::max(Smax, int(jw[m] + Jrow - 1));
  }
  P.Smax = Smax;
  P.tu = make_tiling(rq.Nu, rq.tile);
  P.tv = make_tiling(rq.Nv, rq.tile);
  if (rq.Nu < Smax || rq.Nv < Smax)
    throw std::invalid_argument("grid is smaller than the largest w-projection support");
  for (int b = 0; b < P.tu.n; ++b)
    if (P.tu.start[b + 1] - P.tu.start[b] < Smax - 1)
      throw std::invalid_argument("grid width is too small for the w-projection support");
  for (int b = 0; b < P.tv.n; ++b)
    if (P.tv.start[b + 1] - P.tv.start[b] < Smax - 1)
      throw std::invalid_argument("grid height is too small for the w-projection support");
  const int ntu = P.tu.n, ntv = P.tv.n, ntiles = ntu * ntv;

  // The kernel sees w - mean(w) (operators.h:323).
  double wmean = 0;
  if (!rq.plain) {
    for (int64_t m = 0; m < M; ++m) wmean += rq.w[m];
    if (M > 0) wmean /= double(M);
  }
  auto w_of = [&](int64_t m) { return rq.plain ? 0.0 : rq.w[m] - wmean; };

  // Placement per row (operators.cc:85-96): kw = floor(u - S/2), taps at
  // kw + 1 .. kw + S (mod N); the phase (-1)^(kw_u + kw_v) goes with the weight.
  std::vector<int32_t> tile(M), local(M);
  std::vector<uint8_t> flip(M);
  for (int64_t m = 0; m < M; ++m) {
    const int S = jw[m] + Jrow - 1;
    const double kwu = std::floor(rq.u[m] - S * 0.5), kwv = std::floor(rq.v[m] - S * 0.5);
    const int q0 = int(wrap(kwu + 1, rq.Nu)), p0 = int(wrap(kwv + 1, rq.Nv));
    const int a = P.tv.of[p0], b = P.tu.of[q0];
    tile[m] = a * ntu + b;
    local[m] = ((p0 - P.tv.start[a]) << 8) | (q0 - P.tu.start[b]);
    flip[m] = uint8_t((int64_t(kwu) + int64_t(kwv)) & 1);
  }
  // Plan order: tile, then support descending (warps take visibilities in
  // turn, so neighbours in this order cost about the same), then caller order.
  std::vector<int32_t> order(M);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
    if (tile[x] != tile[y]) return tile[x] < tile[y];
    return jw[x] > jw[y];
  });
  P.du_lambda = pixel_to_lambda(rq.cellx, rq.imsizex, rq.oversample_ratio);
  P.dv_lambda = pixel_to_lambda(rq.celly, rq.imsizey, rq.oversample_ratio);
  P.code.resize(M);
  P.factor.resize(M);
  P.weight.resize(M);
  P.slot_user.resize(M);
  P.user_slot.resize(M);
  int64_t off = 0;
  for (int64_t i = 0; i < M; ++i) {
    const int32_t m = order[i];
    const int S = jw[m] + Jrow - 1;
    const int lp = local[m] >> 8, lq = local[m] & 0xff;  // item_pack layout below
    // plain rows: one term (the separable taps)
    const int terms =
        rq.plain ? 1 : row_terms(rq.u[m], rq.v[m], w_of(m), jw[m], P.du_lambda, P.dv_lambda);
    P.code[i] = lp | (lq << 8) | (S << 16) | (terms << 24);
    P.factor[i] = off;
    off += int64_t(2) * wrow_rank(P.code[i]) * S;
    const std::complex<double> wgt = rq.weights ? rq.weights[m] : std::complex<double>(1.0, 0.0);
    P.weight[i] = flip[m] ? -wgt : wgt;
    P.slot_user[i] = m;
    P.user_slot[m] = int32_t(i);
    P.taps += int64_t(S) * S;
  }
  P.factor_count = off;
  P.kernel = rq.kernel;
  P.oversample_ratio = rq.oversample_ratio;
  P.gen_u.resize(M);
  P.gen_v.resize(M);
  P.gen_w.resize(M);
  P.gen_jw.resize(M);
  for (int64_t i = 0; i < M; ++i) {
    const int32_t m = order[i];
    P.gen_u[i] = rq.u[m];
    P.gen_v[i] = rq.v[m];
    P.gen_w[i] = w_of(m);
    P.gen_jw[i] = jw[m];
  }

  // Tasks: consecutive visibilities of one tile, bounded in taps.
  P.tile_tasks.assign(ntiles + 1, 0);
  int64_t i = 0;
  for (int t = 0; t < ntiles; ++t) {
    const int a = t / ntu, b = t % ntu;
    int64_t e = i;
    while (e < M && tile[order[e]] == t) ++e;
    int64_t s = i;
    while (s < e) {
      int64_t k = s, taps = 0;
      while (k < e && (k == s || taps + wrow_taps(P.code[k]) <= rq.max_taps_per_task)) {
        taps += wrow_taps(P.code[k]);
        ++k;
      }
      Task tk{};
      tk.P = P.tv.start[a];
      tk.Q = P.tu.start[b];
      tk.H = P.tv.start[a + 1] - P.tv.start[a];
      tk.W = P.tu.start[b + 1] - P.tu.start[b];
      tk.batch_begin = int32_t(s);
      tk.batch_end = int32_t(k);
      tk.tile = t;
      P.tasks.push_back(tk);
      s = k;
    }
    P.tile_tasks[t + 1] = int32_t(P.tasks.size());
    P.win_rows = std::max(P.win_rows, P.tv.start[a + 1] - P.tv.start[a] + Smax - 1);
    P.win_cols = std::max(P.win_cols, P.tu.start[b + 1] - P.tu.start[b] + Smax - 1);
    i = e;
  }
  // Staging chunks (the factor ranges of consecutive rows are contiguous).
  P.chunk_values = std::max(kWChunkValues, 6 * Smax);
  P.task_chunk.assign(P.tasks.size() + 1, 0);
  for (size_t k = 0; k < P.tasks.size(); ++k) {
    const int32_t b = P.tasks[k].batch_begin, e = P.tasks[k].batch_end;
    auto fend = [&](int32_t r) { return r + 1 < M ? P.factor[r + 1] : P.factor_count; };
    for (int32_t r = b; r < e;) {
      WChunk c{P.factor[r], fend(r), r, r + 1};
      while (c.vis_end < e && c.vis_end - c.vis_begin < kWChunkVis &&
             fend(c.vis_end) - c.fbegin <= P.chunk_values) {
        c.fend = fend(c.vis_end);
        ++c.vis_end;
      }
      P.chunks.push_back(c);
      r = c.vis_end;
    }
    P.task_chunk[k + 1] = int32_t(P.chunks.size());
  }
  // Launch order: longest tasks (in taps) first while the grid stays in L2,
  // else the spatial order (see build_plan).
  P.task_order.resize(P.tasks.size());
  std::iota(P.task_order.begin(), P.task_order.end(), 0);
  if (int64_t(rq.Nu) * rq.Nv * 8 <= kLptGridBytes) {
    std::vector<int64_t> cost(P.tasks.size(), 0);
    for (size_t k = 0; k < P.tasks.size(); ++k)
      for (int i = P.tasks[k].batch_begin; i < P.tasks[k].batch_end; ++i) {
        cost[k] += wrow_taps(P.code[i]);
      }
    std::stable_sort(P.task_order.begin(), P.task_order.end(),
                     [&](int32_t x, int32_t y) { return cost[x] > cost[y]; });
  }
  return P;
}

template <typename T>
void wplan_factors(const WPlan &P, int64_t i0, int64_t i1, std::complex<T> *out) {
  const int J = P.J;
  const GriddingKernel kern(P.kernel, J, P.oversample_ratio);
  // plain rows: details::init_gridding_matrix_2d receives (kernelv, kernelu)
  // in its (u, v) slots (operators.h:322-324), so the u-axis taps use the
  // kernel of support Jv and the v-axis taps the kernel of support Ju
  const GriddingKernel kern_uslot(P.kernel, P.plain ? P.Jv : J, P.oversample_ratio);
  const GriddingKernel kern_vslot(P.kernel, P.plain ? P.Ju : J, P.oversample_ratio);
  const double dul = P.du_lambda, dvl = P.dv_lambda;
  const int64_t base = i0 < int64_t(P.factor.size()) ? P.factor[i0] : 0;
#pragma omp parallel
  {
    std::vector<double> fu(J), fv(J);
    std::vector<std::complex<double>> alpha(3 * 256), beta(3 * 256), row(6 * 256);
#pragma omp for schedule(dynamic, 1024)
    for (int64_t i = i0; i < i1; ++i) {
      const double u = P.gen_u[i], v = P.gen_v[i], w = P.gen_w[i];
      if (P.plain) {
        // operators.cc:8-46: taps at k + 1 .. k + Ju with k = floor(u - Ju / 2),
        // which sit at offset k - kw inside the row of S = J cells placed at
        // kw = floor(u - S / 2); zero elsewhere; the phase (-1)^j as below
        const int S = J;
        const double kwu = std::floor(u - S * 0.5), kwv = std::floor(v - S * 0.5);
        const double ku = std::floor(u - P.Ju * 0.5), kv = std::floor(v - P.Jv * 0.5);
        const int ou = int(ku - kwu), ov = int(kv - kwv);
        for (int k = 0; k < 2 * S; ++k) row[k] = 0.0;
        for (int j = 1; j <= P.Jv; ++j) row[ov + j - 1] = kern_vslot.value(v - (kv + j));
        for (int j = 1; j <= P.Ju; ++j) row[S + ou + j - 1] = kern_uslot.value(u - (ku + j));
        std::complex<T> *dst = out + (P.factor[i] - base);
        for (int r = 0; r < 2; ++r)
          for (int k = 0; k < S; ++k) {
            const std::complex<double> z = (k & 1) ? -row[r * S + k] : row[r * S + k];
            dst[r * S + k] = std::complex<T>(T(z.real()), T(z.imag()));
          }
        continue;
      }
      const int Jw = P.gen_jw[i], S = Jw + J - 1;
      // Kaiser-Bessel (or other) taps: projection_kernels.cc:66-75
      const double du = u - std::floor(u - J * 0.5), dv = v - std::floor(v - J * 0.5);
      for (int k = 0; k < J; ++k) {
        fu[k] = kern.value(du - k - 1);
        fv[k] = kern.value(dv - k - 1);
      }
      // w-kernel samples: sample (row jv, column ju) = kernelw(dwu - ju - 1,
      // dwv - jv - 1, w) (projection_kernels.cc:76-82, 31-47)
      const double dwu = u - std::floor(u - Jw * 0.5), dwv = v - std::floor(v - Jw * 0.5);
      std::complex<double> *a1 = &alpha[0], *a2 = &alpha[256], *a3 = &alpha[512];
      std::complex<double> *b1 = &beta[0], *b2 = &beta[256], *b3 = &beta[512];
      const std::complex<double> c = std::complex<double>(1.0 / w, 0.0) / std::complex<double>(0, 1);
      // g = (a~ / (w i)) b~^T + (1 - chi_v) 1^T + chi_v (1 - chi_u)^T: every
      // sample comes from exactly one term, so no term cancels another.
      for (int k = 0; k < Jw; ++k) {
        const double U = dwu - k - 1, V = dwv - k - 1;
        const bool ok_u = std::abs(U * dul / w) < 1, ok_v = std::abs(V * dvl / w) < 1;
        const double uu = U * dul, vv = V * dvl;
        a1[k] = ok_v ? c * std::exp(std::complex<double>(0, -kPi * vv * vv / w)) : 0.0;
        b1[k] = ok_u ? std::exp(std::complex<double>(0, -kPi * uu * uu / w)) : 0.0;
        a2[k] = ok_v ? 0.0 : 1.0;
        b2[k] = 1.0;
        a3[k] = ok_v ? 1.0 : 0.0;
        b3[k] = ok_u ? 0.0 : 1.0;
      }
      // the nonzero terms only (the row code's term mask): A of each, then B
      const int terms = wrow_terms(P.code[i]), rank = wrow_rank(P.code[i]);
      int e = 0;
      for (int r = 0; r < 3; ++r)
        if (terms >> r & 1) {
          conv1d(fv.data(), J, &alpha[256 * r], Jw, &row[e * S]);
          conv1d(fu.data(), J, &beta[256 * r], Jw, &row[(rank + e) * S]);
          ++e;
        }
      std::complex<T> *dst = out + (P.factor[i] - base);
      for (int r = 0; r < 2 * rank; ++r)
        for (int k = 0; k < S; ++k) {
          const std::complex<double> z = (k & 1) ? -row[r * S + k] : row[r * S + k];
          dst[r * S + k] = std::complex<T>(T(z.real()), T(z.imag()));
        }
    }
  }
}

template void wplan_factors<float>(const WPlan &, int64_t, int64_t, std::complex<float> *);
template void wplan_factors<double>(const WPlan &, int64_t, int64_t, std::complex<double> *);

}  // namespace pg
