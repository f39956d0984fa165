// extern "C" boundary: translates pg::Error into status codes and a
// thread-local message; nothing throws across it.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/purify_gb300.h"
#include "batch.h"
#include "gridding_kernels.h"
#include "ingest.h"
#include "operator.h"
#include "plan.h"
#include "psf.h"
#include "server.h"
#include "solver.h"
#include "wplan.h"

struct purify_gb300_operator {
  std::unique_ptr<pg::Operator> impl;
};
struct purify_gb300_plan {
  pg::Plan plan;
};
struct purify_gb300_walk_plan {
  pg::WalkPlan plan;
  int ntu = 0, ntv = 0;
};
struct purify_gb300_psf {
  std::unique_ptr<pg::PsfConvolve> impl;
};
struct purify_gb300_server {
  std::unique_ptr<pg::Server> impl;
};
struct purify_gb300_batch {
  std::unique_ptr<pg::Batch> impl;
  pg::BatchTuning tuning;
  int nch = 0;
};

namespace {
thread_local std::string g_last_error;

template <class F>
int guard(F &&f) {
  try {
    g_last_error.clear();
    f();
    return PURIFY_GB300_OK;
  } catch (const pg::Error &e) {
    g_last_error = e.what();
    return int(e.status);
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return PURIFY_GB300_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return PURIFY_GB300_INTERNAL;
  }
}

int null_arg(const char *what) {
  g_last_error = std::string(what) + " is null";
  return PURIFY_GB300_INVALID_ARGUMENT;
}
}  // namespace

extern "C" {

const char *purify_gb300_last_error(void) { return g_last_error.c_str(); }
const char *purify_gb300_version(void) { return "purify_gb300 0.1.0 (sm_103a)"; }

void purify_gb300_default_args(purify_gb300_create_args *a) {
  if (!a) return;
  std::memset(a, 0, sizeof(*a));
  a->oversample_ratio = 2.0;
  a->power_iters = 100;
  a->power_tol = 1e-4;
  a->kernel = PURIFY_GB300_KERNEL_KB;
  a->Ju = 4;
  a->Jv = 4;
  a->w_term = 0;
  a->Jw = 6;
  a->cellx = 1.0;
  a->celly = 1.0;
  a->precision = PURIFY_GB300_FP32;
  a->device = 0;
}

int purify_gb300_operator_create(const purify_gb300_create_args *a, purify_gb300_operator **out) {
  return purify_gb300_operator_create_tuned(a, nullptr, out);
}

}  // extern "C"

namespace {
pg::OperatorConfig to_config(const purify_gb300_create_args *a, const purify_gb300_tuning *t) {
  pg::OperatorConfig c;
  c.u = a->u;
  c.v = a->v;
  c.w = a->w;
  c.weights = a->weights;
  c.M = a->M;
  c.imsizey = int(a->imsizey);
  c.imsizex = int(a->imsizex);
  c.oversample_ratio = a->oversample_ratio;
  c.power_iters = int(a->power_iters);
  c.power_tol = a->power_tol;
  c.kernel = a->kernel;
  c.Ju = int(a->Ju);
  c.Jv = int(a->Jv);
  c.w_term = a->w_term != 0;
  c.Jw = int(a->Jw);
  c.jw_rows = a->jw_rows;
  c.cellx = a->cellx;
  c.celly = a->celly;
  c.fp64 = a->precision == PURIFY_GB300_FP64;
  c.device = a->device;
  if (t) {
    c.threads = t->threads;
    c.max_per_item = t->max_per_item;
    c.tile = t->tile;
    c.fused_permute = t->fused_permute;
    c.cell_group = t->cell_group;
    c.class_cap = t->class_cap;
    c.keep_store = t->keep_store;
    c.fft_columns = t->fft_columns;
    c.grid_walk = t->grid_walk;
    c.normal_pass = t->normal_pass;
  }
  if (a->precision != PURIFY_GB300_FP32 && a->precision != PURIFY_GB300_FP64)
    throw pg::Error(pg::kInvalidArgument, "unknown precision");
  return c;
}
}  // namespace

extern "C" {

int purify_gb300_operator_create_tuned(const purify_gb300_create_args *a,
                                       const purify_gb300_tuning *t,
                                       purify_gb300_operator **out) {
  if (!a) return null_arg("args");
  if (!out) return null_arg("out");
  *out = nullptr;
  return guard([&] {
    const pg::OperatorConfig c = to_config(a, t);
    auto *h = new purify_gb300_operator();
    try {
      h->impl = pg::Operator::create(c);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int purify_gb300_operator_destroy(purify_gb300_operator *op) {
  return guard([&] { delete op; });
}

int purify_gb300_forward(purify_gb300_operator *op, const void *x, void *y, void *stream) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    if ((!x && i.imsizex * int64_t(i.imsizey) > 0) || (!y && i.M > 0))
      throw pg::Error(pg::kInvalidArgument, "null buffer");
    op->impl->forward(x, y, static_cast<cudaStream_t>(stream));
  });
}
int purify_gb300_adjoint(purify_gb300_operator *op, const void *y, void *x, void *stream) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    if ((!x && i.imsizex * int64_t(i.imsizey) > 0) || (!y && i.M > 0))
      throw pg::Error(pg::kInvalidArgument, "null buffer");
    op->impl->adjoint(y, x, static_cast<cudaStream_t>(stream));
  });
}
int purify_gb300_normal(purify_gb300_operator *op, const void *x, void *out, void *stream) {
  if (!op) return null_arg("operator");
  if (!x || !out) return null_arg("buffer");
  return guard([&] { op->impl->normal(x, out, static_cast<cudaStream_t>(stream)); });
}
void purify_gb300_fb_default_params(purify_gb300_fb_params *p) {
  if (!p) return;
  const pg::FbParams d;
  p->iterations = uint32_t(d.iterations);
  p->step = d.step;
  p->gamma_scale = d.gamma_scale;
  p->update_scale = d.update_scale;
  p->update_tol = d.update_tol;
  p->update_iters = uint32_t(d.update_iters);
  p->real_constraint = d.real_constraint ? 1 : 0;
  p->positive_constraint = d.positive_constraint ? 1 : 0;
}
int purify_gb300_forward_backward(purify_gb300_operator *op, const void *y, void *x,
                                  const purify_gb300_fb_params *params, double *gammas,
                                  void *stream) {
  if (!op) return null_arg("operator");
  if (!params) return null_arg("params");
  if (!x || (!y && op->impl->info().M > 0)) return null_arg("buffer");
  return guard([&] {
    pg::FbParams p;
    p.iterations = int(params->iterations);
    p.step = params->step;
    p.gamma_scale = params->gamma_scale;
    p.update_scale = params->update_scale;
    p.update_tol = params->update_tol;
    p.update_iters = int(params->update_iters);
    p.real_constraint = params->real_constraint != 0;
    p.positive_constraint = params->positive_constraint != 0;
    pg::forward_backward(*op->impl, y, x, p, gammas, static_cast<cudaStream_t>(stream));
  });
}
int purify_gb300_psf_create(purify_gb300_operator *op, uint32_t power_iters, double power_tol,
                            purify_gb300_psf **out) {
  if (!op) return null_arg("operator");
  if (!out) return null_arg("out");
  *out = nullptr;
  return guard([&] {
    std::unique_ptr<purify_gb300_psf> h(new purify_gb300_psf);
    h->impl = pg::PsfConvolve::create(*op->impl, int(power_iters), power_tol);
    *out = h.release();
  });
}
int purify_gb300_psf_apply(purify_gb300_psf *p, const void *x, void *out, void *stream) {
  if (!p) return null_arg("psf");
  if (!x || !out) return null_arg("buffer");
  return guard([&] { p->impl->apply(x, out, static_cast<cudaStream_t>(stream)); });
}
int purify_gb300_psf_norm(const purify_gb300_psf *p, double *norm) {
  if (!p) return null_arg("psf");
  if (!norm) return null_arg("norm");
  *norm = p->impl->norm();
  return PURIFY_GB300_OK;
}
int purify_gb300_psf_destroy(purify_gb300_psf *p) {
  return guard([&] { delete p; });
}

int purify_gb300_degrid(purify_gb300_operator *op, const void *grid, void *vis, void *stream) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    if (!grid || (!vis && i.M > 0)) throw pg::Error(pg::kInvalidArgument, "null buffer");
    op->impl->degrid(grid, vis, static_cast<cudaStream_t>(stream));
  });
}
int purify_gb300_grid(purify_gb300_operator *op, const void *vis, void *grid, void *stream) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    if (!grid || (!vis && i.M > 0)) throw pg::Error(pg::kInvalidArgument, "null buffer");
    op->impl->grid(vis, grid, static_cast<cudaStream_t>(stream));
  });
}
// G^H for callers that may not allocate: scratch from the library's fixed
// device array (see no_alloc.cu).
int purify_gb300_grid_no_alloc(purify_gb300_operator *op, const void *vis, void *grid,
                               void *stream) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    if (!grid || (!vis && i.M > 0)) throw pg::Error(pg::kInvalidArgument, "null buffer");
    op->impl->grid_no_alloc(vis, grid, static_cast<cudaStream_t>(stream));
  });
}
int purify_gb300_grid_no_alloc_bytes(const purify_gb300_operator *op, int64_t *bytes) {
  if (!op) return null_arg("operator");
  if (!bytes) return null_arg("bytes");
  return guard([&] { *bytes = op->impl->no_alloc_bytes(); });
}
int purify_gb300_wrow_taps(double u, double v, double w_centered, uint32_t Jw, uint32_t J,
                           int32_t kernel, double os, uint32_t imsizey, uint32_t imsizex,
                           double cellx, double celly, double *out) {
  if (!out) return null_arg("out");
  return guard([&] {
    // two rows with w and -w: their mean is 0, so row 0 sees w_centered
    const double uu[2] = {u, u}, vv[2] = {v, v}, ww[2] = {w_centered, -w_centered};
    pg::WPlanRequest rq;
    rq.u = uu;
    rq.v = vv;
    rq.w = ww;
    rq.M = 2;
    rq.Nu = int(std::floor(imsizex * os));
    rq.Nv = int(std::floor(imsizey * os));
    rq.imsizex = int(imsizex);
    rq.imsizey = int(imsizey);
    rq.oversample_ratio = os;
    rq.cellx = cellx;
    rq.celly = celly;
    rq.J = int(J);
    rq.Jw = int(Jw);
    rq.kernel = kernel;
    pg::WPlan p;
    try {
      p = pg::build_wplan(rq);
    } catch (const std::invalid_argument &e) {
      throw pg::Error(pg::kInvalidArgument, e.what());
    }
    const int64_t i = p.user_slot[0];
    const int S = pg::wrow_support(p.code[i]), rank = pg::wrow_rank(p.code[i]);
    std::vector<std::complex<double>> f(2 * rank * S);
    pg::wplan_factors<double>(p, i, i + 1, f.data());
    const std::complex<double> sgn = p.weight[i];  // +-1: (-1)^(kw_u + kw_v)
    for (int jv = 0; jv < S; ++jv)
      for (int ju = 0; ju < S; ++ju) {
        std::complex<double> k = 0;
        for (int r = 0; r < rank; ++r) k += f[r * S + jv] * f[(rank + r) * S + ju];
        k *= sgn;
        out[2 * (jv * S + ju)] = k.real();
        out[2 * (jv * S + ju) + 1] = k.imag();
      }
  });
}

int purify_gb300_correction(int32_t kernel, uint32_t Ju, uint32_t Jv, uint32_t imsizey,
                            uint32_t imsizex, double os, double *S_out) {
  if (!S_out) return null_arg("S_out");
  return guard([&] {
    const std::string why = pg::check_kernel_request(kernel, int(Ju), int(Jv));
    if (!why.empty()) throw pg::Error(pg::kInvalidArgument, why);
    if (imsizey == 0 || imsizex == 0 || !(os > 0))
      throw pg::Error(pg::kInvalidArgument, "empty image or bad oversampling");
    std::vector<double> S(size_t(imsizey) * imsizex);
    pg::correction_factors(kernel, int(Ju), int(Jv), int(imsizey), int(imsizex), os, S.data());
    for (size_t k = 0; k < S.size(); ++k) {
      S_out[2 * k] = S[k];
      S_out[2 * k + 1] = 0.0;
    }
  });
}
int purify_gb300_stage_timing(purify_gb300_operator *op, int enable) {
  if (!op) return null_arg("operator");
  return guard([&] { op->impl->set_stage_timing(enable != 0); });
}
int purify_gb300_stage_times(purify_gb300_operator *op, double *total_ms, int64_t *launches) {
  if (!op) return null_arg("operator");
  return guard([&] { op->impl->stage_times(total_ms, launches); });
}
int purify_gb300_forward_host(purify_gb300_operator *op, const double *x, double *y) {
  if (!op) return null_arg("operator");
  return guard([&] { op->impl->forward_host(x, y); });
}
int purify_gb300_adjoint_host(purify_gb300_operator *op, const double *y, double *x) {
  if (!op) return null_arg("operator");
  return guard([&] { op->impl->adjoint_host(y, x); });
}
int purify_gb300_power_method(purify_gb300_operator *op, uint32_t iters, double tol,
                              double *norm_out) {
  if (!op) return null_arg("operator");
  return guard([&] {
    const double n = op->impl->power_method(int(iters), tol);
    if (norm_out) *norm_out = n;
  });
}
int purify_gb300_set_norm(purify_gb300_operator *op, double norm) {
  if (!op) return null_arg("operator");
  return guard([&] { op->impl->set_norm(norm); });
}
int purify_gb300_get_norm(const purify_gb300_operator *op, double *norm) {
  if (!op) return null_arg("operator");
  if (!norm) return null_arg("norm");
  return guard([&] { *norm = op->impl->norm(); });
}
int purify_gb300_operator_info(const purify_gb300_operator *op, purify_gb300_info *info) {
  if (!op) return null_arg("operator");
  if (!info) return null_arg("info");
  return guard([&] {
    const pg::OperatorInfo i = op->impl->info();
    info->M = i.M;
    info->imsizey = uint32_t(i.imsizey);
    info->imsizex = uint32_t(i.imsizex);
    info->ftsizev = uint32_t(i.ftsizev);
    info->ftsizeu = uint32_t(i.ftsizeu);
    info->Ju = uint32_t(i.Ju);
    info->Jv = uint32_t(i.Jv);
    info->precision = i.fp64 ? PURIFY_GB300_FP64 : PURIFY_GB300_FP32;
    info->kernel = i.kernel;
    info->w_term = i.w_term ? 1 : 0;
    info->nnz = i.nnz;
    info->occupied_cells = i.occupied_cells;
    info->work_items = i.work_items;
    info->tasks = i.tasks;
    info->device_bytes = i.device_bytes;
    info->kernel_fit_error = i.kernel_fit_error;
    info->norm = i.norm;
    info->slots = i.slots;
    info->window_cells = i.window_cells;
    info->factor_values = i.factor_values;
    info->cell_group = i.cell_group;
    info->walk_tasks = i.walk_tasks;
    info->walk_steps = i.walk_steps;
  });
}

// utilities::set_cell_size (utilities.cc:208-256) then uv_scale
// (utilities.cc:258-278) for coordinates given in wavelengths.
int purify_gb300_lambda_to_pixels(const double *u, const double *v, int64_t M, double cellx,
                                  double celly, uint32_t ftsizeu, uint32_t ftsizev,
                                  double *u_out, double *v_out) {
  if (M > 0 && (!u || !v || !u_out || !v_out)) return null_arg("coordinate buffer");
  return guard([&] {
    constexpr double pi = 3.14159265358979323846;
    double mu = 0, mv = 0;
    for (int64_t m = 0; m < M; ++m) {
      mu = std::max(mu, u[m] * u[m]);
      mv = std::max(mv, v[m] * v[m]);
    }
    double cu = cellx, cv = celly;
    if (cu == 0 && cv == 0) {
      cu = (180 * 3600) / std::sqrt(mu) / pi / 3;
      cv = (180 * 3600) / std::sqrt(mv) / pi / 3;
    }
    if (cv == 0) cv = cu;
    const double su = 180 * 3600 / cu / pi, sv = 180 * 3600 / cv / pi;
    for (int64_t m = 0; m < M; ++m) {
      const double ur = u[m] / su * 2 * pi, vr = v[m] / sv * 2 * pi;
      u_out[m] = ur / (2 * pi) * ftsizeu;
      v_out[m] = vr / (2 * pi) * ftsizev;
    }
  });
}

int purify_gb300_uv_to_pixels(const double *u, const double *v, int64_t M, int32_t units,
                              double cellx, double celly, uint32_t ftsizeu, uint32_t ftsizev,
                              double *u_out, double *v_out) {
  if (M > 0 && (!u || !v || !u_out || !v_out)) return null_arg("coordinate buffer");
  switch (units) {
    case PURIFY_GB300_UNITS_LAMBDA:
      return purify_gb300_lambda_to_pixels(u, v, M, cellx, celly, ftsizeu, ftsizev, u_out, v_out);
    case PURIFY_GB300_UNITS_RADIANS:
      // uv_scale alone (utilities.cc:258-278)
      return guard([&] {
        constexpr double pi = 3.14159265358979323846;
        for (int64_t m = 0; m < M; ++m) {
          u_out[m] = u[m] / (2 * pi) * ftsizeu;
          v_out[m] = v[m] / (2 * pi) * ftsizev;
        }
      });
    case PURIFY_GB300_UNITS_PIXELS:
      return guard([&] {
        for (int64_t m = 0; m < M; ++m) {
          u_out[m] = u[m];
          v_out[m] = v[m];
        }
      });
    default:
      return guard([&] {
        throw pg::Error(pg::kInvalidArgument,
                        "unknown visibility units " + std::to_string(units) +
                            " (0 lambda, 1 radians, 2 pixels)");
      });
  }
}

int purify_gb300_plan_create(const double *u, const double *v, const double *weights, int64_t M,
                             uint32_t ftsizeu, uint32_t ftsizev, uint32_t J,
                             purify_gb300_plan **out) {
  return purify_gb300_plan_create_grouped(u, v, weights, M, ftsizeu, ftsizev, J, 1, out);
}
int purify_gb300_plan_create_grouped(const double *u, const double *v, const double *weights,
                                     int64_t M, uint32_t ftsizeu, uint32_t ftsizev, uint32_t J,
                                     int32_t group, purify_gb300_plan **out) {
  if (!out) return null_arg("out");
  *out = nullptr;
  return guard([&] {
    pg::PlanRequest rq;
    rq.u = u;
    rq.v = v;
    rq.weights = reinterpret_cast<const std::complex<double> *>(weights);
    rq.M = M;
    rq.Nu = int(ftsizeu);
    rq.Nv = int(ftsizev);
    rq.Ju = rq.Jv = int(J);
    rq.group = group;
    auto *p = new purify_gb300_plan();
    try {
      p->plan = pg::build_plan(rq);
    } catch (const std::invalid_argument &e) {
      delete p;
      throw pg::Error(pg::kInvalidArgument, e.what());
    }
    *out = p;
  });
}

int purify_gb300_plan_sizes(const purify_gb300_plan *p, int64_t *sizes) {
  if (!p || !sizes) return null_arg("plan or sizes");
  const pg::Plan &P = p->plan;
  sizes[0] = P.M;
  sizes[1] = P.S;
  sizes[2] = int64_t(P.batch_base.size());
  sizes[3] = int64_t(P.tasks.size());
  sizes[4] = P.tu.n;
  sizes[5] = P.tv.n;
  sizes[6] = P.win_rows;
  sizes[7] = P.win_cols;
  sizes[8] = P.unit_weights ? 1 : 0;
  sizes[9] = P.group;
  sizes[10] = P.win_stride;
  return PURIFY_GB300_OK;
}

int purify_gb300_plan_export(const purify_gb300_plan *p, double *frac, double *weight,
                             int32_t *slot_user, int32_t *user_slot, int32_t *batches,
                             int32_t *lane_code, int32_t *tasks, int32_t *tile_tasks,
                             int32_t *tu_start, int32_t *tv_start) {
  if (!p) return null_arg("plan");
  const pg::Plan &P = p->plan;
  for (int64_t s = 0; s < P.S; ++s) {
    if (frac) {
      frac[2 * s] = P.frac_u[s];
      frac[2 * s + 1] = P.frac_v[s];
    }
    if (weight) {
      std::complex<double> w;
      if (P.unit_weights)
        w = P.slot_user[s] < 0 ? 0.0 : (P.flip[s] ? -1.0 : 1.0);
      else
        w = P.weight[s];
      weight[2 * s] = w.real();
      weight[2 * s + 1] = w.imag();
    }
    if (slot_user) slot_user[s] = P.slot_user[s];
  }
  if (user_slot) std::copy(P.user_slot.begin(), P.user_slot.end(), user_slot);
  for (size_t b = 0; b < P.batch_base.size(); ++b)
    if (batches) {
      batches[2 * b] = P.batch_base[b];
      batches[2 * b + 1] = P.batch_kmax[b];
    }
  if (lane_code) std::copy(P.lane_code.begin(), P.lane_code.end(), lane_code);
  if (tasks)
    for (size_t k = 0; k < P.tasks.size(); ++k) {
      const pg::Task &t = P.tasks[k];
      const int32_t row[8] = {t.P, t.Q, t.H, t.W, t.batch_begin, t.batch_end, t.tile, 0};
      std::memcpy(tasks + 8 * k, row, sizeof(row));
    }
  if (tile_tasks) std::copy(P.tile_tasks.begin(), P.tile_tasks.end(), tile_tasks);
  if (tu_start) std::copy(P.tu.start.begin(), P.tu.start.end(), tu_start);
  if (tv_start) std::copy(P.tv.start.begin(), P.tv.start.end(), tv_start);
  return PURIFY_GB300_OK;
}

int purify_gb300_plan_destroy(purify_gb300_plan *p) {
  delete p;
  return PURIFY_GB300_OK;
}

int purify_gb300_walk_plan_create(const double *u, const double *v, int64_t M, uint32_t ftsizeu,
                                  uint32_t ftsizev, uint32_t J, purify_gb300_walk_plan **out) {
  if (!out) return null_arg("out");
  *out = nullptr;
  if (M > 0 && (!u || !v)) return null_arg("u / v");
  return guard([&] {
    pg::PlanRequest rq;
    rq.u = u;
    rq.v = v;
    rq.M = M;
    rq.Nu = int(ftsizeu);
    rq.Nv = int(ftsizev);
    rq.Ju = rq.Jv = int(J);
    std::unique_ptr<purify_gb300_walk_plan> p(new purify_gb300_walk_plan);
    try {
      p->plan = pg::build_walk_plan(rq);
    } catch (const std::invalid_argument &e) {
      throw pg::Error(pg::kInvalidArgument, e.what());
    }
    p->ntu = pg::make_tiling(rq.Nu, rq.tile).n;
    p->ntv = pg::make_tiling(rq.Nv, rq.tile).n;
    *out = p.release();
  });
}
int purify_gb300_walk_plan_sizes(const purify_gb300_walk_plan *p, int64_t *sizes) {
  if (!p) return null_arg("plan");
  if (!sizes) return null_arg("sizes");
  const pg::WalkPlan &W = p->plan;
  const int64_t s[8] = {W.M, int64_t(W.tasks.size()), p->ntu, p->ntv, W.win_rows, W.win_cols,
                        W.win_stride, W.steps};
  std::copy(s, s + 8, sizes);
  return PURIFY_GB300_OK;
}
int purify_gb300_walk_plan_export(const purify_gb300_walk_plan *p, double *frac,
                                  int32_t *slot_user, int32_t *counts, int32_t *colstart,
                                  int32_t *tasks, int32_t *task_order, int32_t *tile_tasks) {
  if (!p) return null_arg("plan");
  const pg::WalkPlan &W = p->plan;
  for (int64_t s = 0; s < W.M; ++s) {
    if (frac) {
      frac[2 * s] = W.flip[s] ? -W.frac_u[s] : W.frac_u[s];
      frac[2 * s + 1] = W.frac_v[s];
    }
    if (slot_user) slot_user[s] = W.slot_user[s];
  }
  if (counts) std::copy(W.counts.begin(), W.counts.end(), counts);
  if (colstart) std::copy(W.colstart.begin(), W.colstart.end(), colstart);
  if (tasks)
    for (size_t k = 0; k < W.tasks.size(); ++k) {
      const pg::Task &t = W.tasks[k];
      const int32_t row[8] = {t.P, t.Q, t.H, t.W, 0, 0, t.tile, 0};
      std::copy(row, row + 8, tasks + 8 * k);
    }
  if (task_order) std::copy(W.task_order.begin(), W.task_order.end(), task_order);
  if (tile_tasks) std::copy(W.tile_tasks.begin(), W.tile_tasks.end(), tile_tasks);
  return PURIFY_GB300_OK;
}
int purify_gb300_walk_plan_destroy(purify_gb300_walk_plan *p) {
  delete p;
  return PURIFY_GB300_OK;
}

int purify_gb300_kernel_taps(int32_t kernel, uint32_t J, double os, int32_t precision,
                             const double *t, int64_t n, double *out, double *fit_error) {
  return guard([&] {
    const std::string why = pg::check_kernel_request(kernel, int(J), int(J));
    if (!why.empty()) throw pg::Error(pg::kInvalidArgument, why);
    if (J < 1 || J > pg::kMaxJ) throw pg::Error(pg::kUnsupported, "support out of range");
    const bool f64 = precision == PURIFY_GB300_FP64;
    const int nc = f64 ? pg::kCoefF64 : pg::kCoefF32;
    const pg::GriddingKernel k(kernel, int(J), os);
    const pg::AxisFit fit = pg::fit_axis(k, int(J), nc);
    if (fit_error) *fit_error = fit.max_error;
    for (int64_t q = 0; q < n; ++q) {
      if (f64) {
        pg::eval_taps<double>(fit, int(J), t[q], out + q * J);
      } else {
        float kf[pg::kMaxJ];
        pg::eval_taps<float>(fit, int(J), t[q], kf);
        for (uint32_t j = 0; j < J; ++j) out[q * J + j] = kf[j];
      }
    }
  });
}

int purify_gb300_batch_create(const purify_gb300_channel *channels, int32_t nch,
                              double oversample_ratio, int32_t kernel, uint32_t J,
                              int32_t precision, int32_t device,
                              const purify_gb300_batch_tuning *tuning, purify_gb300_batch **out) {
  if (!out) return null_arg("out");
  if (!channels) return null_arg("channels");
  return guard([&] {
    if (nch < 1) throw pg::Error(pg::kInvalidArgument, "a batch needs at least one channel");
    if (precision != PURIFY_GB300_FP32 && precision != PURIFY_GB300_FP64)
      throw pg::Error(pg::kInvalidArgument, "unknown precision");
    pg::BatchConfig cfg;
    cfg.channels.resize(nch);
    for (int c = 0; c < nch; ++c) {
      pg::ChannelSpec &s = cfg.channels[c];
      s.u = channels[c].u;
      s.v = channels[c].v;
      s.weights = reinterpret_cast<const std::complex<double> *>(channels[c].weights);
      s.M = channels[c].M;
      s.imsizey = int(channels[c].imsizey);
      s.imsizex = int(channels[c].imsizex);
    }
    cfg.oversample_ratio = oversample_ratio;
    cfg.kernel = kernel;
    cfg.J = int(J);
    cfg.fp64 = precision == PURIFY_GB300_FP64;
    cfg.device = device;
    pg::BatchTuning t;
    if (tuning) {
      t.tile = tuning->tile > 0 ? tuning->tile : pg::kTile;
      t.max_per_item = tuning->max_per_item > 0 ? tuning->max_per_item : 16;
      t.degrid_threads = tuning->degrid_threads > 0 ? tuning->degrid_threads : 128;
      t.grid_threads = tuning->grid_threads > 0 ? tuning->grid_threads : 128;
      t.cell_group = tuning->cell_group > 0 ? tuning->cell_group : 1;
      t.fft_columns = tuning->fft_columns;
    } else {
      t = pg::autotune_batch(cfg);
    }
    cfg.tile = t.tile;
    cfg.cell_group = t.cell_group;
    cfg.fft_columns = t.fft_columns;
    cfg.max_per_item = t.max_per_item;
    cfg.threads = 128;
    cfg.degrid_threads = t.degrid_threads;
    cfg.grid_threads = t.grid_threads;
    std::unique_ptr<purify_gb300_batch> b(new purify_gb300_batch);
    b->impl = pg::Batch::create(cfg);
    b->tuning = t;
    b->nch = nch;
    *out = b.release();
  });
}
int purify_gb300_batch_destroy(purify_gb300_batch *b) {
  delete b;
  return PURIFY_GB300_OK;
}
int purify_gb300_batch_get_tuning(const purify_gb300_batch *b, purify_gb300_batch_tuning *t) {
  if (!b) return null_arg("batch");
  if (!t) return null_arg("tuning");
  t->tile = b->tuning.tile;
  t->max_per_item = b->tuning.max_per_item;
  t->degrid_threads = b->tuning.degrid_threads;
  t->grid_threads = b->tuning.grid_threads;
  t->cell_group = b->tuning.cell_group;
  t->fft_columns = b->tuning.fft_columns;
  return PURIFY_GB300_OK;
}
int purify_gb300_batch_bind(purify_gb300_batch *b, const void *const *x_in, void *const *vis,
                            void *const *x_out, void *stream) {
  if (!b) return null_arg("batch");
  return guard([&] { b->impl->bind(x_in, vis, x_out, static_cast<cudaStream_t>(stream)); });
}
int purify_gb300_batch_apply(purify_gb300_batch *b, int32_t directions, void *stream) {
  if (!b) return null_arg("batch");
  return guard([&] { b->impl->apply(directions, static_cast<cudaStream_t>(stream)); });
}
int purify_gb300_batch_power_method(purify_gb300_batch *b, uint32_t iters, double tol,
                                    double *norms) {
  if (!b) return null_arg("batch");
  return guard([&] { b->impl->power_method(int(iters), tol, norms); });
}
int purify_gb300_batch_set_norms(purify_gb300_batch *b, const double *norms) {
  if (!b) return null_arg("batch");
  if (!norms) return null_arg("norms");
  return guard([&] { b->impl->set_norms(norms); });
}
int purify_gb300_batch_get_norms(const purify_gb300_batch *b, double *norms) {
  if (!b) return null_arg("batch");
  if (!norms) return null_arg("norms");
  b->impl->get_norms(norms);
  return PURIFY_GB300_OK;
}
int purify_gb300_batch_time(purify_gb300_batch *b, int32_t what, uint32_t reps, double *ms) {
  if (!b) return null_arg("batch");
  if (!ms) return null_arg("ms");
  return guard([&] { *ms = b->impl->time_apply(what, int(reps)); });
}
int purify_gb300_batch_info_get(const purify_gb300_batch *b, purify_gb300_batch_info *info) {
  if (!b) return null_arg("batch");
  if (!info) return null_arg("info");
  const pg::BatchInfo i = b->impl->info();
  info->channels = i.channels;
  info->size_groups = i.size_groups;
  info->visibilities = i.visibilities;
  info->pixels = i.pixels;
  info->tasks = i.tasks;
  info->device_bytes = i.device_bytes;
  return PURIFY_GB300_OK;
}

int purify_gb300_server_create(const purify_gb300_server_config *cfg, purify_gb300_server **out) {
  if (!cfg) return null_arg("config");
  if (!out) return null_arg("out");
  *out = nullptr;
  return guard([&] {
    pg::ServerConfig c;
    c.device = cfg->device;
    c.slots = cfg->slots;
    c.hbm_budget = cfg->hbm_budget_bytes;
    c.norm_slots = cfg->norm_slots;
    std::unique_ptr<purify_gb300_server> h(new purify_gb300_server);
    h->impl.reset(new pg::Server(c));
    *out = h.release();
  });
}
int purify_gb300_server_destroy(purify_gb300_server *s) {
  return guard([&] { delete s; });
}
int purify_gb300_server_add_coverage(purify_gb300_server *s, const purify_gb300_create_args *a,
                                     int32_t *coverage) {
  if (!s) return null_arg("server");
  if (!a) return null_arg("args");
  if (!coverage) return null_arg("coverage");
  return guard([&] { *coverage = s->impl->add_coverage(to_config(a, nullptr)); });
}
}  // extern "C"

namespace {
pg::Request to_request(const purify_gb300_request *rq) {
  pg::Request r;
  r.coverage = rq->coverage;
  r.kind = rq->kind;
  r.x_in = rq->x_in;
  r.vis_in = rq->vis_in;
  r.vis_out = rq->vis_out;
  r.x_out = rq->x_out;
  r.iters = int(rq->iters);
  r.tol = rq->tol;
  return r;
}
}  // namespace

extern "C" {
int purify_gb300_server_submit(purify_gb300_server *s, const purify_gb300_request *rq,
                               int64_t *ticket) {
  if (!s) return null_arg("server");
  if (!rq) return null_arg("request");
  if (!ticket) return null_arg("ticket");
  return guard([&] { *ticket = s->impl->submit(to_request(rq)); });
}
int purify_gb300_server_wait(purify_gb300_server *s, int64_t ticket, double timeout_s,
                             purify_gb300_result *out) {
  if (!s) return null_arg("server");
  int rc = PURIFY_GB300_OK;
  const int g = guard([&] {
    pg::RequestResult r;
    if (!s->impl->wait(ticket, timeout_s, &r)) {
      rc = PURIFY_GB300_TIMEOUT;
      return;
    }
    if (out) {
      out->status = r.status;
      out->iterations = r.iterations;
      out->norm = r.norm;
      out->queue_ms = r.queue_ms;
      out->run_ms = r.run_ms;
      out->latency_ms = r.latency_ms;
      out->device_bytes = r.device_bytes;
    }
  });
  if (g != PURIFY_GB300_OK) return g;
  if (rc == PURIFY_GB300_TIMEOUT) g_last_error = "request still running";
  return rc;
}
int purify_gb300_server_request_bytes(const purify_gb300_server *s, const purify_gb300_request *rq,
                                      int64_t *bytes) {
  if (!s) return null_arg("server");
  if (!rq) return null_arg("request");
  if (!bytes) return null_arg("bytes");
  return guard([&] { *bytes = s->impl->request_bytes(to_request(rq)); });
}
int purify_gb300_server_get_stats(const purify_gb300_server *s, purify_gb300_server_stats *out) {
  if (!s) return null_arg("server");
  if (!out) return null_arg("stats");
  const pg::ServerStats t = s->impl->stats();
  out->submitted = t.submitted;
  out->completed = t.completed;
  out->rejected = t.rejected;
  out->failed = t.failed;
  out->inflight_peak = t.inflight_peak;
  out->bytes_peak = t.bytes_peak;
  out->bytes_budget = t.bytes_budget;
  out->latency_p50_ms = t.latency_p50_ms;
  out->latency_p99_ms = t.latency_p99_ms;
  out->latency_mean_ms = t.latency_mean_ms;
  out->visibility_passes = t.visibility_passes;
  return PURIFY_GB300_OK;
}

int purify_gb300_vis_file_rows(const char *path, int64_t *rows) {
  if (!path) return null_arg("path");
  if (!rows) return null_arg("rows");
  return guard([&] { *rows = pg::vis_file_rows(path); });
}
int purify_gb300_read_visibility(const char *path, int32_t w_term, int64_t rows, double *u,
                                 double *v, double *w, double *vis, double *weights) {
  if (!path) return null_arg("path");
  if (!u || !v || !vis || !weights) return null_arg("output");
  if (w_term && !w) return null_arg("w");
  return guard([&] {
    pg::read_visibility(path, w_term != 0, rows, u, v, w,
                        reinterpret_cast<std::complex<double> *>(vis),
                        reinterpret_cast<std::complex<double> *>(weights));
  });
}
int purify_gb300_init_weights(const double *u, const double *v, const double *weights, int64_t M,
                              double oversample_factor, int32_t weighting, double R,
                              uint32_t ftsizeu, uint32_t ftsizev, int32_t device, double *out) {
  if (M > 0 && (!u || !v || !weights || !out)) return null_arg("buffer");
  return guard([&] {
    pg::init_weights(u, v, reinterpret_cast<const std::complex<double> *>(weights), M,
                     oversample_factor, weighting, R, int(ftsizeu), int(ftsizev), device,
                     reinterpret_cast<std::complex<double> *>(out));
  });
}

}  // extern "C"
