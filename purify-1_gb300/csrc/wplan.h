// Coverage plan of the w-projection operator (host, FP64).
//
// Each visibility m has its own kernel row K_m of S_m x S_m taps, S_m = Jw_m +
// J - 1, the Kaiser-Bessel taps linearly convolved with Jw_m x Jw_m samples of
// the w-kernel (cpp/purify/projection_kernels.cc:59-85, operators.cc:49-99).
// The sample matrix of w_projection_kernel_approx is exp(-i pi (U^2+V^2)/w) /
// (w i) on the rectangle where |U/w| < 1 and |V/w| < 1 and 1 elsewhere
// (projection_kernels.cc:16-47), so it has rank at most 3:
//   g = (a~ / (w i)) b~^T + (1 - chi_v) 1^T + chi_v (1 - chi_u)^T
// (a~, b~ the masked 1-D chirps, chi the validity masks; every sample comes
// from exactly one term, so no term cancels another in finite precision).
// The convolution is bilinear, so K_m = sum_r A_r B_r^T with up to six
// length-S factor vectors, which is what is stored (FP64-generated, in the
// operator's precision).  Terms whose masks make them zero are not stored:
// where the validity rectangle covers all of a row's samples K_m has rank 1.
#pragma once
#include <complex>
#include <cstdint>
#include <vector>

#include "plan.h"

namespace pg {

struct WPlanRequest {
  const double *u = nullptr, *v = nullptr, *w = nullptr;  // pixels, pixels, wavelengths
  const std::complex<double> *weights = nullptr;
  const int32_t *jw_rows = nullptr;  // per-row w-support, or null for Jw everywhere
  int64_t M = 0;
  int Nu = 0, Nv = 0, imsizex = 0, imsizey = 0;
  double oversample_ratio = 2.0, cellx = 1.0, celly = 1.0;
  int J = 4, Jw = 6;
  int kernel = kKB;
  int tile = kTile;
  int64_t max_taps_per_task = 1 << 18;
  // Plain separable rows (no w-term): each row is the Ju u-axis taps times
  // the Jv v-axis taps, placed as details::init_gridding_matrix_2d places
  // them (operators.cc:8-46) inside a square row of S = max(Ju, Jv) cells,
  // rank 1.  Used for supports above the register-block kernels' limit and
  // for Ju != Jv.  w and Jw are ignored.
  bool plain = false;
  int Ju = 4, Jv = 4;
};

struct WPlan {
  int64_t M = 0;
  int Nu = 0, Nv = 0, J = 0, Smax = 0;
  bool plain = false;  // plain separable rows (WPlanRequest::plain)
  int Ju = 0, Jv = 0;
  AxisTiling tu, tv;
  // per visibility in plan order (tile, then support descending)
  std::vector<int32_t> code;     // lp | lq << 8 | S << 16 | terms << 24 (see wrow_terms)
  std::vector<int64_t> factor;   // offset of the row's factors, in complex values
  std::vector<std::complex<double>> weight;  // weight with (-1)^(kw_u + kw_v) folded in
  std::vector<int32_t> slot_user, user_slot;
  int64_t factor_count = 0;  // complex values of all rows' factors
  // generation inputs per visibility in plan order
  std::vector<double> gen_u, gen_v, gen_w;  // w already minus mean(w)
  std::vector<int32_t> gen_jw;
  int kernel = kKB;
  double oversample_ratio = 2.0, du_lambda = 0.0, dv_lambda = 0.0;
  std::vector<Task> tasks;  // batch_begin / batch_end = visibility range in plan order
  std::vector<int32_t> task_order;  // launch order: by decreasing taps, or tile order (see plan.h)
  std::vector<int32_t> tile_tasks;
  // Staging chunks of the G^H kernel: task k owns chunks
  // [task_chunk[k], task_chunk[k + 1]), each at most kWChunkVis rows and
  // chunk_values factor values (plus one value of alignment slack).
  std::vector<WChunk> chunks;
  std::vector<int32_t> task_chunk;
  int chunk_values = 0;
  int win_rows = 0, win_cols = 0;
  int64_t taps = 0;  // sum of S^2
};

WPlan build_wplan(const WPlanRequest &rq);

// Fields of a row code: the support S and the mask of stored terms (bit r:
// term r of the sample matrix is nonzero); the rank is the mask's popcount.
inline int wrow_support(int32_t code) { return (code >> 16) & 0xff; }
inline int wrow_terms(int32_t code) { return (code >> 24) & 7; }
inline int wrow_rank(int32_t code) {
  const int t = wrow_terms(code);
  return (t & 1) + ((t >> 1) & 1) + ((t >> 2) & 1);
}
inline int64_t wrow_taps(int32_t code) {
  const int64_t S = wrow_support(code);
  return S * S;
}

// Factors of rows [i0, i1) of the plan, FP64-generated, written in T to
// out[factor[i] - factor[i0] ...]: per row A_0..A_{rank-1} then
// B_0..B_{rank-1} over the row's nonzero terms (S complex each, (-1)^j of the
// phase folded in) with K = sum_r A_r B_r^T.
template <typename T>
void wplan_factors(const WPlan &plan, int64_t i0, int64_t i1, std::complex<T> *out);

}  // namespace pg
