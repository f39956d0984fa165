#include "operator.h"

#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <vector>

#include "device_kernels.h"
#include "device_util.h"
#include "fft_kernels.h"
#include "gridding_kernels.h"
#include "no_alloc.h"
#include "plan.h"
#include "wkernels.h"
#include "wplan.h"

namespace pg {

// t + d (t in [0, 1), d the visibility's cell inside its group) in the
// operator's precision.  Rounding must not carry t up to the next cell: the
// kernels read d back as the integer part, so a value that rounds to d + 1
// is stored as the largest value below it.
template <typename real>
real fraction_in_cell(double x) {
  const double d = std::floor(x);
  const real r = real(x);
  return double(r) >= d + 1 ? std::nextafter(real(d + 1), real(0)) : r;
}
template float fraction_in_cell<float>(double);
template double fraction_in_cell<double>(double);

namespace {
// The column walk of G^H: CTA size (4 warps, a quarter of the tile's columns
// each), and the fullest base cell it takes (one lane walks a cell's
// visibilities alone; a coverage with fuller cells keeps the work items,
// which split a cell over several lanes).
// Supports from which the default launch shape and adjoint path change
// (see the constructor).
constexpr int kWideSupport = 6;
// Supports from which the adjoint's grid kernel gathers caller order itself
// by default.
constexpr int kGatherInGridSupport = 4;
// Launch shape of normal_kernel: two warps per CTA.  Its two register
// blocks per lane leave room for few warps, and its shared memory holds the
// grid window besides the warp windows.
constexpr LaunchShape kNormalShape{64};
// Host entry points of FP32 operators: the c128 <-> c64 conversion and the
// host copies run in up to kCopyChunks chunks of at least kCopyChunkMin
// values, overlapped (upload_c128, download_c128).
constexpr int kCopyChunks = 8;
constexpr int64_t kCopyChunkMin = int64_t(1) << 18;
constexpr int kWalkThreads = 128;
constexpr int kWalkMaxCellCount = 256;
}  // namespace

void cuda_check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation)
    throw Error(kOutOfMemory, std::string(what) + ": " + cudaGetErrorString(e));
  throw Error(kCudaError, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

// Largest caller-ordered visibility vector the adjoint's gather keeps in L2
// at evict-last priority: three quarters of the GB300's 126 MB L2, so the
// other streams of a step keep some room (the 10^7-visibility FP32 vector is
// 80 MB).
constexpr int64_t kKeepVisL2Bytes = int64_t(96) << 20;

template <typename real>
class OperatorT final : public Operator {
 public:
  explicit OperatorT(const OperatorConfig &cfg);
  ~OperatorT() override;
  void forward(const void *x, void *y, cudaStream_t stream) override;
  void adjoint(const void *y, void *x, cudaStream_t stream) override;
  void normal(const void *x, void *out, cudaStream_t stream) override;
  void degrid(const void *grid, void *vis, cudaStream_t stream) override;
  void grid(const void *vis, void *grid, cudaStream_t stream) override;
  void grid_no_alloc(const void *vis, void *grid, cudaStream_t stream) override;
  int64_t no_alloc_bytes() const override;
  void forward_host(const double *x, double *y) override;
  void adjoint_host(const double *y, double *x) override;
  double power_method(int iters, double tol) override;
  void set_norm(double norm) override;
  double norm() const override { return norm_; }
  OperatorInfo info() const override { return info_; }
  void set_stage_timing(bool on) override;
  void stage_times(double *total_ms, int64_t *launches) override;
  WorkspaceSizes workspace_sizes() const override;
  void forward_ws(const void *x, void *y, const Workspace &ws) override;
  void adjoint_ws(const void *y, void *x, const Workspace &ws) override;
  void power_ws(void *x, int first, int count, double *sq, double *partial,
                const Workspace &ws) override;
  bool needs_column_plan() const override { return fused_fft_ && !own_cols_; }

 private:
  enum Stage { kPad = 0, kFftF, kDegrid, kGrid, kFold, kFftI, kCrop, kCompact, kExpand };
  // Events bracketing one stage launch; recorded only while timing is on.
  void mark_begin(int stage);
  void mark_end(int stage);
  void drain_timing();
  struct Mark {
    int stage;
    cudaEvent_t a, b;
  };
  bool timing_ = false;
  std::vector<Mark> marks_;
  std::vector<cudaEvent_t> event_pool_;
  size_t marks_used_ = 0;
  double stage_ms_[kStages] = {};
  int64_t stage_n_[kStages] = {};
  using C = std::complex<real>;
  void forward_on_stream(const void *x, void *y);
  void adjoint_on_stream(const void *y, void *x);
  // G and G^H between the grid and the slot-ordered visibility buffer.
  void degrid_slots(const void *grid, void *caller_vis = nullptr);
  void grid_slots(void *grid, const void *caller_vis = nullptr);
  void grid_core(void *grid, const void *vis, const int32_t *slot_user, void *windows);
  void fold_into(void *grid, const void *windows);
  void degrid_on_stream(const void *grid, void *y);
  void grid_on_stream(const void *y, void *grid);
  // Phi' / Phi'^H with visibilities kept in slot order (power method).
  FftArgs fft_args() const;
  void forward_slots(const void *x, void *caller_vis = nullptr);
  void adjoint_slots(void *x, const void *caller_vis = nullptr, bool walk = false);
  // G^H of the column-walk plan: ws->slots (walk order) -> task windows -> grid
  void walk_grid(void *grid);
  void fold_into(void *grid, const void *windows, const int32_t *tile_tasks);
  // Phi'^H Phi' x with the visibilities kept in slot order between G and G^H
  // (power method, normal operator); the weights' conjugates are applied there.
  void normal_slots(const void *x, void *out);
  // F Z S x into ws->work; S^H Z^H F^H of ws->work into x
  void forward_grid(const void *x);
  void inverse_grid(void *x);
  // Slot-ordered weights for the gather before G^H, or null for unit weights.
  const void *slot_weights() const { return split_weights_ ? weight_.get() : nullptr; }
  void join(cudaStream_t user);
  void release(cudaStream_t user);
  void upload_correction();
  void ensure_host_staging();
  // Host complex<double> vector <-> device vector of the operator's type
  // through the c128 staging buffer `stage`, in chunks: the conversion
  // kernels run on stream_ and the copies on copy_stream_, so that each
  // chunk's conversion overlaps the copies of the others.
  void upload_c128(const double *host, void *stage, void *dev, int64_t n);
  void download_c128(const void *dev, void *stage, double *host, int64_t n);
  cudaStream_t copy_stream_ = nullptr;
  std::vector<cudaEvent_t> copy_ev_;

  OperatorInfo info_;
  int device_ = 0;
  int Nx_ = 0, Ny_ = 0, Nu_ = 0, Nv_ = 0, x0_ = 0, y0_ = 0, J_ = 0;
  int64_t M_ = 0, N_ = 0, S_ = 0;
  bool wmode_ = false;  // row-factor kernels (w-projection rows, or plain rows)
  bool rows_mode_ = false;  // plain separable rows on the row-factor kernels
  // halo of the task windows + 1 along u and v (J plus the group's extra
  // cell, or the largest w support)
  int fold_J_ = 0, fold_Jv_ = 0;
  DeviceBuffer wcode_, wfactor_, wfactors_, wchunks_, wtask_chunk_;
  int wchunk_values_ = 0;
  int64_t nnz_ = 0, occupied_ = 0, work_items_ = 0, factor_values_ = 0;
  void init_plain(const OperatorConfig &cfg, int64_t &bytes, AxisTiling &tu, AxisTiling &tv,
                  std::vector<int32_t> &tile_tasks);
  void init_w(const OperatorConfig &cfg, int64_t &bytes, AxisTiling &tu, AxisTiling &tv,
              std::vector<int32_t> &tile_tasks);
  bool unit_weights_ = true;
  // Weights (plain rows): the gridding kernels have no weight stream (the
  // phase sign rides in t_u) and the weights are applied around them: in
  // caller order after G (wcaller_), conjugated in slot order before G^H
  // (weight_; by the gather where there is one).
  bool split_weights_ = false;
  DeviceBuffer wcaller_;  // caller-ordered weights
  bool fused_forward_ = true, fused_adjoint_ = false;
  // The adjoint's gather keeps the caller-ordered visibilities in L2
  // (evict-last) when they fit in kKeepVisL2Bytes: in a forward / adjoint
  // loop the next degrid's scattered stores into them then hit L2.  Only on
  // the operator's own scratch: applies on other workspaces run concurrently
  // (the server), and several kept vectors would crowd each other out.
  bool keep_vis_l2_ = false;
  // degrid stores the caller-ordered output at evict-last priority too
  bool keep_store_ = false;
  double norm_ = 1.0;
  std::vector<double> su_, sv_;  // 1 / ft kernel at the image pixels (unscaled)
  std::vector<real> su_scaled_, sv_real_;
  PolyTable<real> poly_{};
  LaunchShape shape_;
  int ntasks_ = 0, win_rows_ = 0, win_cols_ = 0, win_stride_ = 0, ntu_ = 0, ntv_ = 0;
  int group_ = 1;  // cells per work item along each axis (plan's group)
  int64_t slot_stride_ = 0;

  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_in_ = nullptr, ev_out_ = nullptr;
  cufftHandle fft_ = 0;
  bool fft_ok_ = false;
  // FP32 with a power-of-two grid width: fused row passes + a cuFFT column
  // transform (fft_kernels.h) replace Z S + 2-D FFT and 2-D FFT + S^H Z^H.
  bool fused_fft_ = false;
  cufftHandle fft_cols_ = 0;
  DeviceBuffer tw_u_;
  // own_cols_: the column transforms run as the library's column pass
  // (launch_fft_cols); otherwise through the workspace's cuFFT column plan
  bool own_cols_ = false;
  // Phi^H Phi's G^H G by normal_kernel in one pass (tuning normal_pass = 1;
  // unit weights, FP32, single-cell items, J <= 6) instead of degrid then
  // grid through the slot buffer.
  bool one_pass_normal_ = false;
  // Column-walk plan of G^H (used by Phi^H from caller order when walk_)
  bool walk_ = false;
  int walk_ntasks_ = 0, walk_win_rows_ = 0, walk_win_stride_ = 0, walk_max_steps_ = 0;
  int64_t walk_steps_ = 0;
  DeviceBuffer walk_frac_, walk_user_, walk_weight_, walk_counts_, walk_colstart_, walk_tasks_,
      walk_order_, walk_tile_tasks_;
  DeviceBuffer tw_v_;
  bool use_fused_fft() const { return fused_fft_ && (own_cols_ || ws_->fft_cols != 0); }
  FftColArgs col_args(const void *in, void *out) const;
  std::mutex mu_;

  DeviceBuffer task_order_, frac_, weight_, slot_user_, user_slot_, batches_, lane_code_, tasks_, tile_tasks_,
      tu_start_, tv_start_, tu_of_, tv_of_, su_d_, sv_d_, pad_, work_, tilebuf_, slots_,
      norm_partial_, norm_out_;
  DeviceBuffer x128_, y128_, xc_, yc_, pm_x_;
  bool staging_ = false, pm_ready_ = false;
  // Scratch of the apply being enqueued: the operator's own (own_) or a
  // caller's workspace (the *_ws entry points).
  Workspace own_;
  const Workspace *ws_ = &own_;
  DeviceBuffer su_unit_d_;  // correction scaled for norm 1 (Phi')
  const real *su_active() const {
    return ws_->unit_norm ? su_unit_d_.as<real>() : su_d_.as<real>();
  }
  void with_workspace(const Workspace &ws, const std::function<void()> &f);
  // Recorded applies on the operator's own scratch (see run_recorded).
  using GraphKey = std::tuple<int, const void *, const void *>;
  std::map<GraphKey, cudaGraphExec_t> graphs_;
  std::set<GraphKey> seen_;
  void run_recorded(int kind, const void *in, void *out, const std::function<void()> &enqueue);
  void drop_graphs();
};

template <typename real>
OperatorT<real>::OperatorT(const OperatorConfig &cfg) {
  device_ = cfg.device;
  DeviceGuard guard(device_);
  Nx_ = cfg.imsizex;
  Ny_ = cfg.imsizey;
  Nu_ = int(std::floor(cfg.imsizex * cfg.oversample_ratio));
  Nv_ = int(std::floor(cfg.imsizey * cfg.oversample_ratio));
  x0_ = int(std::floor(Nu_ * 0.5 - Nx_ * 0.5));
  y0_ = int(std::floor(Nv_ * 0.5 - Ny_ * 0.5));
  J_ = cfg.Ju;
  M_ = cfg.M;
  N_ = int64_t(Nx_) * Ny_;

  // Kernel state, FP64 fit.  The reference builds G with (kernelv, kernelu)
  // in its (u, v) slots (operators.h:322-324); with Ju == Jv both are the same
  // function, which is the only case accepted here.
  // Supports above the register-block kernels' limit, and Ju != Jv, run as
  // plain rows on the row-factor kernels (see WPlanRequest::plain).
  rows_mode_ = !cfg.w_term && (cfg.Ju != cfg.Jv || cfg.Ju > kMaxJ);
  wmode_ = cfg.w_term || rows_mode_;
  GriddingKernel kern(cfg.kernel, J_, cfg.oversample_ratio);
  const int nc = PolyCount<real>::value;
  AxisFit fit;
  std::memset(&poly_, 0, sizeof(poly_));
  if (!wmode_) {
    fit = fit_axis(kern, J_, nc);
    for (int j = 0; j < J_; ++j)
      for (int s = 0; s < fit.nsub; ++s)
        for (int k = 0; k < nc; ++k) {
          const real c = real(fit.coef[(size_t(j) * fit.nsub + s) * nc + k]);
          poly_.u.c[j][s][k] = c;
          poly_.v.c[j][s][k] = c;
        }
    poly_.nsub_u = poly_.nsub_v = fit.nsub;
  }

  // Gridding correction S(j, i) = 1 / (ftv(y0 + j + 0.5) ftu(x0 + i + 0.5))
  // (operators.cc:101-121; the w = 0 chirp times Nx Ny is 1), ftu of support
  // Ju along x and ftv of support Jv along y (create_kernels, kernels.cc:
  // 233-323).
  const GriddingKernel kern_x(cfg.kernel, cfg.Ju, cfg.oversample_ratio);
  const GriddingKernel kern_y(cfg.kernel, cfg.Jv, cfg.oversample_ratio);
  su_.resize(Nx_);
  sv_.resize(Ny_);
  for (int i = 0; i < Nx_; ++i)
    su_[i] = 1.0 / kern_x.correction((x0_ + i + 0.5) / Nu_ - 0.5);
  for (int j = 0; j < Ny_; ++j)
    sv_[j] = 1.0 / kern_y.correction((y0_ + j + 0.5) / Nv_ - 0.5);

  // Defaults measured on the 10^7-visibility workload (1024^2 image, KB,
  // FP32).  Wide supports (J >= 6): 64-thread CTAs, and the adjoint's grid
  // kernel gathers caller order itself; its per-visibility work hides the
  // gathers' latency (J = 6: step 0.414 ms; 128 threads 0.423; a separate
  // gather 0.47).  Narrower supports: 128-thread CTAs.  From J = 4 the grid
  // kernel gathers caller order with four steps of loads in flight and the
  // indices three steps ahead (GridAhead; J = 4: adjoint 0.213 ms against
  // 0.221 with the separate gather, J = 5: 0.233 against 0.241).  Below
  // J = 4 the steps are too short and the adjoint gathers into slot order
  // first (J = 2: adjoint 0.209 ms against 0.294).  The forward always
  // writes caller order directly (scattered stores) unless the tuning asks
  // for the slot-ordered path.  The w-projection kernels always use the
  // slot-ordered buffer.
  const bool wide = J_ >= kWideSupport;
  shape_.threads = cfg.threads > 0 ? cfg.threads : (wide ? 64 : 128);
  fused_forward_ = !wmode_ && cfg.fused_permute != 0;
  keep_vis_l2_ = int64_t(sizeof(C)) * M_ <= kKeepVisL2Bytes;
  keep_store_ = cfg.keep_store != 0;
  fused_adjoint_ = !wmode_ && (cfg.fused_permute == 1 ||
                               (cfg.fused_permute < 0 && J_ >= kGatherInGridSupport));

  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_in_, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_out_, cudaEventDisableTiming), "cudaEventCreate");

  int64_t bytes = 0;
  AxisTiling tu, tv;
  std::vector<int32_t> tile_tasks;
  if (wmode_)
    init_w(cfg, bytes, tu, tv, tile_tasks);
  else
    init_plain(cfg, bytes, tu, tv, tile_tasks);
  // split weights are applied to the slot-ordered buffer before G^H, and the
  // column walk reads its own slot order
  if (split_weights_ || walk_) fused_adjoint_ = false;
  ntu_ = tu.n;
  ntv_ = tv.n;
  slot_stride_ = int64_t(win_rows_) * win_cols_;
  if (!wmode_) {
    // Shared memory of the largest launch this operator makes (windows,
    // batch headers, per-warp staging in the most demanding layout).
    int optin = 0;
    cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_),
               "cudaDeviceGetAttribute");
    const int nsub = std::max(poly_.nsub_u, poly_.nsub_v);
    const size_t need = std::max(
        degrid_smem_bytes(sizeof(real), J_, win_rows_, win_cols_, shape_, true, group_, nsub),
        grid_smem_bytes(sizeof(real), J_, win_rows_, win_cols_, shape_, true, group_, nsub));
    if (need > size_t(optin))
      throw Error(kUnsupported, "tile / threads / support need " + std::to_string(need) +
                                    " bytes of shared memory per CTA; the device allows " +
                                    std::to_string(optin));
    const size_t nsm =
        normal_smem_bytes(sizeof(real), J_, win_rows_, win_cols_, kNormalShape, group_, nsub);
    const bool want = cfg.normal_pass == 1 || (cfg.normal_pass == 0 && J_ < kWideSupport);
    one_pass_normal_ = want && !split_weights_ && nsm > 0 && nsm <= size_t(optin);
  }
  {
    tile_tasks_.alloc(sizeof(int32_t) * tile_tasks.size(), &bytes);
    tile_tasks_.upload(tile_tasks.data(), sizeof(int32_t) * tile_tasks.size(), stream_);
    tu_start_.alloc(sizeof(int32_t) * tu.start.size(), &bytes);
    tu_start_.upload(tu.start.data(), sizeof(int32_t) * tu.start.size(), stream_);
    tv_start_.alloc(sizeof(int32_t) * tv.start.size(), &bytes);
    tv_start_.upload(tv.start.data(), sizeof(int32_t) * tv.start.size(), stream_);
    tu_of_.alloc(sizeof(int32_t) * tu.of.size(), &bytes);
    tu_of_.upload(tu.of.data(), sizeof(int32_t) * tu.of.size(), stream_);
    tv_of_.alloc(sizeof(int32_t) * tv.of.size(), &bytes);
    tv_of_.upload(tv.of.data(), sizeof(int32_t) * tv.of.size(), stream_);
    su_d_.alloc(sizeof(real) * Nx_, &bytes);
    sv_d_.alloc(sizeof(real) * Ny_, &bytes);
    su_unit_d_.alloc(sizeof(real) * Nx_, &bytes);
    const size_t gbytes = sizeof(C) * size_t(Nu_) * Nv_;
    pad_.alloc(gbytes, &bytes);
    cuda_check(cudaMemsetAsync(pad_.get(), 0, gbytes, stream_), "cudaMemset");
    work_.alloc(gbytes, &bytes);
    tilebuf_.alloc(sizeof(C) * size_t(slot_stride_) * std::max(ntasks_, 1), &bytes);
    slots_.alloc(sizeof(C) * std::max<int64_t>(S_, 1), &bytes);
    norm_partial_.alloc(sizeof(double) * kNormBlocks, &bytes);
    norm_out_.alloc(sizeof(double), &bytes);
    // The staging vectors above are pageable; wait before they go out of scope.
    cuda_check(cudaStreamSynchronize(stream_), "upload");
  }
  cufft_check(cufftPlan2d(&fft_, Nv_, Nu_, Traits<real>::kType), "cufftPlan2d");
  fft_ok_ = true;
  if (sizeof(real) == 4 && fft_rows_supported(Nu_)) {
    const std::vector<float> twu = fft_twiddles(Nu_);
    tw_u_.alloc(sizeof(float) * twu.size(), &bytes);
    tw_u_.upload(twu.data(), sizeof(float) * twu.size(), stream_);
    own_cols_ = cfg.fft_columns != 1 && fft_cols_supported(Nv_, Nu_);
    std::vector<float> twv;
    if (own_cols_) {
      twv = fft_twiddles(Nv_);
      tw_v_.alloc(sizeof(float) * twv.size(), &bytes);
      tw_v_.upload(twv.data(), sizeof(float) * twv.size(), stream_);
    } else {
      fft_cols_ = make_column_plan<real>(Nu_, Nv_, stream_, &bytes);
    }
    cuda_check(cudaStreamSynchronize(stream_), "twiddle upload");
    fused_fft_ = true;
  }
  cufft_check(cufftSetStream(fft_, stream_), "cufftSetStream");
  size_t ws = 0;
  if (cufftGetSize(fft_, &ws) == CUFFT_SUCCESS) bytes += int64_t(ws);
  own_.pad = pad_.get();
  own_.work = work_.get();
  own_.tilebuf = tilebuf_.get();
  own_.slots = slots_.get();
  own_.fft = fft_;
  own_.fft_cols = fft_cols_;
  own_.stream = stream_;
  {
    // Phi' (norm 1) correction for power-method workspaces.
    const double c = 1.0 / std::sqrt(double(Nu_) * double(Nv_));
    std::vector<real> su1(Nx_);
    for (int i = 0; i < Nx_; ++i) su1[i] = real(su_[i] * c);
    su_unit_d_.upload(su1.data(), sizeof(real) * Nx_, stream_);
    cuda_check(cudaStreamSynchronize(stream_), "correction upload");
  }

  info_.M = M_;
  info_.device = device_;
  info_.imsizey = Ny_;
  info_.imsizex = Nx_;
  info_.ftsizev = Nv_;
  info_.ftsizeu = Nu_;
  info_.Ju = cfg.Ju;
  info_.Jv = cfg.Jv;
  info_.fp64 = cfg.fp64;
  info_.kernel = cfg.kernel;
  info_.w_term = cfg.w_term;
  info_.tasks = ntasks_;
  info_.device_bytes = bytes;
  info_.kernel_fit_error = wmode_ ? 0.0 : fit.max_error;
  info_.nnz = nnz_;
  info_.occupied_cells = occupied_;
  info_.work_items = work_items_;
  info_.slots = S_;
  info_.window_cells = slot_stride_;
  info_.factor_values = factor_values_;
  info_.cell_group = group_;
  info_.walk_tasks = walk_ ? walk_ntasks_ : 0;
  info_.walk_steps = walk_ ? walk_steps_ : 0;

  set_norm(1.0);
  if (cfg.power_iters > 0) power_method(cfg.power_iters, cfg.power_tol);
}

template <typename real>
void OperatorT<real>::init_plain(const OperatorConfig &cfg, int64_t &bytes, AxisTiling &tu,
                                 AxisTiling &tv, std::vector<int32_t> &tile_tasks) {
  // Coverage plan (FP64 coordinates, tile sort, work items, slots).
  PlanRequest rq;
  rq.u = cfg.u;
  rq.v = cfg.v;
  rq.weights = reinterpret_cast<const std::complex<double> *>(cfg.weights);
  rq.M = cfg.M;
  rq.Nu = Nu_;
  rq.Nv = Nv_;
  rq.Ju = cfg.Ju;
  rq.Jv = cfg.Jv;
  rq.tile = cfg.tile > 0 ? cfg.tile : kTile;
  rq.max_per_item = cfg.max_per_item > 0 ? cfg.max_per_item : 16;
  // Work items of single base cells by default: 2 x 2 groups (a (J + 1)^2
  // block, complex<float> up to kMaxGroupJ) flush fewer blocks but spend
  // more FMAs and registers per visibility, and measured slower on the
  // 10^7-visibility workload (G^H 224 against 172 us, G 160 against 139).
  rq.group = cfg.cell_group == 0 ? 1 : cfg.cell_group;
  rq.class_cap = cfg.class_cap;
  rq.warps = shape_.threads / 32;
  Plan plan;
  try {
    plan = build_plan(rq);
  } catch (const std::invalid_argument &e) {
    throw Error(kInvalidArgument, e.what());
  }
  group_ = plan.group;
  ntasks_ = int(plan.tasks.size());
  win_rows_ = plan.win_rows;
  win_cols_ = plan.win_cols;
  win_stride_ = plan.win_stride;
  // task windows reach a block's extent - 1 cells into the next tiles
  fold_J_ = J_ + group_u(group_) - 1;
  fold_Jv_ = J_ + group_v(group_) - 1;
  S_ = plan.S;
  unit_weights_ = plan.unit_weights;
  split_weights_ = !unit_weights_;
  nnz_ = M_ * int64_t(cfg.Ju) * cfg.Jv;
  occupied_ = plan.occupied_cells;
  work_items_ = int64_t(plan.lane_code.size());
  std::vector<C> fr(S_);
  for (int64_t i = 0; i < S_; ++i) {
    // unit weights: the phase sign (-1)^(k_u + k_v) rides in the sign of t_u
    const real tu = fraction_in_cell<real>(plan.frac_u[i]);
    // the phase sign (-1)^(k_u + k_v) rides in the sign of t_u
    fr[i] = C(plan.flip[i] ? -tu : tu, fraction_in_cell<real>(plan.frac_v[i]));
  }
  frac_.alloc(sizeof(C) * S_, &bytes);
  frac_.upload(fr.data(), sizeof(C) * S_, stream_);
  std::vector<C> wt;
  if (!unit_weights_) {
    wt.resize(S_);
    for (int64_t i = 0; i < S_; ++i) {
      // the sign is in t_u, so this holds the weight itself
      const std::complex<double> w = plan.flip[i] ? -plan.weight[i] : plan.weight[i];
      wt[i] = C(real(w.real()), real(w.imag()));
    }
    weight_.alloc(sizeof(C) * S_, &bytes);
    weight_.upload(wt.data(), sizeof(C) * S_, stream_);
  }
  std::vector<C> wc;
  if (split_weights_) {
    const auto *w = reinterpret_cast<const std::complex<double> *>(cfg.weights);
    wc.resize(M_);
    for (int64_t m = 0; m < M_; ++m) wc[m] = C(real(w[m].real()), real(w[m].imag()));
    wcaller_.alloc(sizeof(C) * std::max<int64_t>(M_, 1), &bytes);
    wcaller_.upload(wc.data(), sizeof(C) * M_, stream_);
  }
  slot_user_.alloc(sizeof(int32_t) * S_, &bytes);
  slot_user_.upload(plan.slot_user.data(), sizeof(int32_t) * S_, stream_);
  user_slot_.alloc(sizeof(int32_t) * M_, &bytes);
  user_slot_.upload(plan.user_slot.data(), sizeof(int32_t) * M_, stream_);
  const size_t nb = plan.batch_base.size();
  std::vector<int2> bt(nb);
  for (size_t k = 0; k < nb; ++k) bt[k] = int2{plan.batch_base[k], plan.batch_kmax[k]};
  batches_.alloc(sizeof(int2) * nb, &bytes);
  batches_.upload(bt.data(), sizeof(int2) * nb, stream_);
  lane_code_.alloc(sizeof(int32_t) * plan.lane_code.size(), &bytes);
  lane_code_.upload(plan.lane_code.data(), sizeof(int32_t) * plan.lane_code.size(), stream_);
  tasks_.alloc(sizeof(Task) * plan.tasks.size(), &bytes);
  tasks_.upload(plan.tasks.data(), sizeof(Task) * plan.tasks.size(), stream_);
  task_order_.alloc(sizeof(int32_t) * plan.task_order.size(), &bytes);
  task_order_.upload(plan.task_order.data(), sizeof(int32_t) * plan.task_order.size(), stream_);
  // the staging vectors are pageable: wait before they go out of scope
  cuda_check(cudaStreamSynchronize(stream_), "upload");
  tu = plan.tu;
  tv = plan.tv;
  tile_tasks = plan.tile_tasks;

  // The column-walk plan of G^H: single-cell items, tiles of at most 32, a
  // support whose J x J register block stays in registers, and no cell so
  // full that one lane would walk it alone for long.
  const int jmax = sizeof(real) == 8 ? 6 : 8;
  WalkPlan wp;
  if (cfg.grid_walk == 1 && group_ == 1 && rq.tile <= 32 && cfg.Ju == cfg.Jv && cfg.Ju <= jmax &&
      M_ > 0 && plan.max_cell_count <= kWalkMaxCellCount) {
    try {
      wp = build_walk_plan(rq);
    } catch (const std::invalid_argument &e) {
      throw Error(kInvalidArgument, e.what());
    }
    int optin = 0;
    cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_),
               "cudaDeviceGetAttribute");
    walk_ = walk_smem_bytes(sizeof(real), wp.win_rows, wp.win_stride,
                            std::max(wp.max_warp_steps, 1), J_,
                            std::max(poly_.nsub_u, poly_.nsub_v)) <= size_t(optin);
  }
  if (walk_) {
    walk_max_steps_ = std::max(wp.max_warp_steps, 1);
    walk_ntasks_ = int(wp.tasks.size());
    walk_win_rows_ = wp.win_rows;
    walk_win_stride_ = wp.win_stride;
    walk_steps_ = wp.steps;
    std::vector<C> wf(M_);
    for (int64_t i = 0; i < M_; ++i) {
      const real tu = fraction_in_cell<real>(wp.frac_u[i]);
      wf[i] = C(wp.flip[i] ? -tu : tu, fraction_in_cell<real>(wp.frac_v[i]));
    }
    walk_frac_.alloc(sizeof(C) * M_, &bytes);
    walk_frac_.upload(wf.data(), sizeof(C) * M_, stream_);
    walk_user_.alloc(sizeof(int32_t) * M_, &bytes);
    walk_user_.upload(wp.slot_user.data(), sizeof(int32_t) * M_, stream_);
    std::vector<C> ww;
    if (split_weights_) {
      // caller weights in walk order, for the gather before G^H
      const auto *w = reinterpret_cast<const std::complex<double> *>(cfg.weights);
      ww.resize(M_);
      for (int64_t s = 0; s < M_; ++s) {
        const std::complex<double> x = w[wp.slot_user[s]];
        ww[s] = C(real(x.real()), real(x.imag()));
      }
      walk_weight_.alloc(sizeof(C) * M_, &bytes);
      walk_weight_.upload(ww.data(), sizeof(C) * M_, stream_);
    }
    walk_counts_.alloc(sizeof(int32_t) * wp.counts.size(), &bytes);
    walk_counts_.upload(wp.counts.data(), sizeof(int32_t) * wp.counts.size(), stream_);
    walk_colstart_.alloc(sizeof(int32_t) * wp.colstart.size(), &bytes);
    walk_colstart_.upload(wp.colstart.data(), sizeof(int32_t) * wp.colstart.size(), stream_);
    walk_tasks_.alloc(sizeof(Task) * wp.tasks.size(), &bytes);
    walk_tasks_.upload(wp.tasks.data(), sizeof(Task) * wp.tasks.size(), stream_);
    walk_order_.alloc(sizeof(int32_t) * wp.task_order.size(), &bytes);
    walk_order_.upload(wp.task_order.data(), sizeof(int32_t) * wp.task_order.size(), stream_);
    walk_tile_tasks_.alloc(sizeof(int32_t) * wp.tile_tasks.size(), &bytes);
    walk_tile_tasks_.upload(wp.tile_tasks.data(), sizeof(int32_t) * wp.tile_tasks.size(), stream_);
    cuda_check(cudaStreamSynchronize(stream_), "upload");
  }
}

template <typename real>
void OperatorT<real>::init_w(const OperatorConfig &cfg, int64_t &bytes, AxisTiling &tu,
                             AxisTiling &tv, std::vector<int32_t> &tile_tasks) {
  WPlanRequest rq;
  rq.u = cfg.u;
  rq.v = cfg.v;
  rq.w = cfg.w;
  rq.weights = reinterpret_cast<const std::complex<double> *>(cfg.weights);
  rq.jw_rows = cfg.jw_rows;
  rq.M = cfg.M;
  rq.Nu = Nu_;
  rq.Nv = Nv_;
  rq.imsizex = Nx_;
  rq.imsizey = Ny_;
  rq.oversample_ratio = cfg.oversample_ratio;
  rq.cellx = cfg.cellx;
  rq.celly = cfg.celly;
  rq.J = cfg.Ju;
  rq.Jw = cfg.Jw;
  rq.kernel = cfg.kernel;
  rq.plain = rows_mode_;
  rq.Ju = cfg.Ju;
  rq.Jv = cfg.Jv;
  // Default tile edge: 24 (measured fastest on the w-projection workload),
  // widened to the largest support - 1 (a window may reach one tile ahead).
  int smax = rows_mode_ ? std::max(cfg.Ju, cfg.Jv) : cfg.Jw + cfg.Ju - 1;
  if (cfg.jw_rows && !rows_mode_) {
    smax = 1;
    for (int64_t m = 0; m < cfg.M; ++m) smax = std::max(smax, cfg.jw_rows[m] + cfg.Ju - 1);
  }
  rq.tile = cfg.tile > 0 ? cfg.tile : std::max(24, smax - 1);
  WPlan plan;
  try {
    plan = build_wplan(rq);
  } catch (const std::invalid_argument &e) {
    throw Error(kInvalidArgument, e.what());
  }
  if (plan.Smax > kMaxWSupport)
    throw Error(kUnsupported, "w-projection support above 32 taps per axis");
  ntasks_ = int(plan.tasks.size());
  win_rows_ = plan.win_rows;
  win_cols_ = plan.win_cols;
  fold_J_ = fold_Jv_ = plan.Smax;
  S_ = M_;
  unit_weights_ = false;
  // the reference's non-zeros (Ju Jv per plain row; the stored rows pad to S^2)
  nnz_ = rows_mode_ ? M_ * int64_t(cfg.Ju) * cfg.Jv : plan.taps;
  occupied_ = 0;
  work_items_ = M_;
  std::vector<C> wt(M_);
  for (int64_t i = 0; i < M_; ++i)
    wt[i] = C(real(plan.weight[i].real()), real(plan.weight[i].imag()));
  weight_.alloc(sizeof(C) * std::max<int64_t>(M_, 1), &bytes);
  weight_.upload(wt.data(), sizeof(C) * M_, stream_);
  wcode_.alloc(sizeof(int32_t) * std::max<int64_t>(M_, 1), &bytes);
  wcode_.upload(plan.code.data(), sizeof(int32_t) * M_, stream_);
  wfactor_.alloc(sizeof(int64_t) * std::max<int64_t>(M_, 1), &bytes);
  wfactor_.upload(plan.factor.data(), sizeof(int64_t) * M_, stream_);
  slot_user_.alloc(sizeof(int32_t) * std::max<int64_t>(M_, 1), &bytes);
  slot_user_.upload(plan.slot_user.data(), sizeof(int32_t) * M_, stream_);
  user_slot_.alloc(sizeof(int32_t) * std::max<int64_t>(M_, 1), &bytes);
  user_slot_.upload(plan.user_slot.data(), sizeof(int32_t) * M_, stream_);
  tasks_.alloc(sizeof(Task) * std::max<size_t>(plan.tasks.size(), 1), &bytes);
  tasks_.upload(plan.tasks.data(), sizeof(Task) * plan.tasks.size(), stream_);
  task_order_.alloc(sizeof(int32_t) * std::max<size_t>(plan.task_order.size(), 1), &bytes);
  task_order_.upload(plan.task_order.data(), sizeof(int32_t) * plan.task_order.size(), stream_);
  wchunks_.alloc(sizeof(WChunk) * std::max<size_t>(plan.chunks.size(), 1), &bytes);
  wchunks_.upload(plan.chunks.data(), sizeof(WChunk) * plan.chunks.size(), stream_);
  wtask_chunk_.alloc(sizeof(int32_t) * plan.task_chunk.size(), &bytes);
  wtask_chunk_.upload(plan.task_chunk.data(), sizeof(int32_t) * plan.task_chunk.size(), stream_);
  wchunk_values_ = plan.chunk_values;
  factor_values_ = plan.factor_count;
  cuda_check(cudaStreamSynchronize(stream_), "upload");
  // Row factors, FP64-generated, uploaded in chunks of rows.  Two values of
  // tail: the G^H staging copies read whole 16-byte pieces.
  wfactors_.alloc(sizeof(C) * (plan.factor_count + 2), &bytes);
  cuda_check(cudaMemset(wfactors_.get(), 0, sizeof(C) * (plan.factor_count + 2)), "memset");
  const int64_t chunk_rows = 1 << 20;
  std::vector<std::complex<real>> buf;
  for (int64_t i0 = 0; i0 < M_; i0 += chunk_rows) {
    const int64_t i1 = std::min(M_, i0 + chunk_rows);
    const int64_t f0 = plan.factor[i0];
    const int64_t f1 = i1 < M_ ? plan.factor[i1] : plan.factor_count;
    buf.resize(size_t(f1 - f0));
    wplan_factors<real>(plan, i0, i1, buf.data());
    cuda_check(cudaMemcpy(wfactors_.as<C>() + f0, buf.data(), sizeof(C) * (f1 - f0),
                          cudaMemcpyHostToDevice),
               "factor upload");
  }
  tu = plan.tu;
  tv = plan.tv;
  tile_tasks = plan.tile_tasks;
}

template <typename real>
OperatorT<real>::~OperatorT() {
  if (stream_) cudaStreamSynchronize(stream_);
  drop_graphs();
  for (cudaEvent_t e : event_pool_) cudaEventDestroy(e);
  if (fft_ok_) cufftDestroy(fft_);
  if (fft_cols_) cufftDestroy(fft_cols_);
  if (ev_in_) cudaEventDestroy(ev_in_);
  if (ev_out_) cudaEventDestroy(ev_out_);
  if (copy_stream_) cudaStreamSynchronize(copy_stream_);
  for (cudaEvent_t e : copy_ev_) cudaEventDestroy(e);
  if (copy_stream_) cudaStreamDestroy(copy_stream_);
  if (stream_) cudaStreamDestroy(stream_);
}

template <typename real>
void OperatorT<real>::upload_correction() {
  // Phi = G F Z S / norm with a unitary F: fold 1 / (sqrt(Nu Nv) norm) into S.
  const double c = 1.0 / (std::sqrt(double(Nu_) * double(Nv_)) * norm_);
  su_scaled_.resize(Nx_);
  sv_real_.resize(Ny_);
  for (int i = 0; i < Nx_; ++i) su_scaled_[i] = real(su_[i] * c);
  for (int j = 0; j < Ny_; ++j) sv_real_[j] = real(sv_[j]);
  su_d_.upload(su_scaled_.data(), sizeof(real) * Nx_, stream_);
  sv_d_.upload(sv_real_.data(), sizeof(real) * Ny_, stream_);
  cuda_check(cudaStreamSynchronize(stream_), "correction upload");
}

template <typename real>
void OperatorT<real>::set_norm(double norm) {
  if (!(norm > 0)) throw Error(kNormNotPositive, "Operator norm is not greater than zero.");
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  norm_ = norm;
  info_.norm = norm;
  upload_correction();
}

template <typename real>
void OperatorT<real>::join(cudaStream_t user) {
  cuda_check(cudaEventRecord(ev_in_, user), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(stream_, ev_in_, 0), "cudaStreamWaitEvent");
}
template <typename real>
void OperatorT<real>::release(cudaStream_t user) {
  cuda_check(cudaEventRecord(ev_out_, stream_), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(user, ev_out_, 0), "cudaStreamWaitEvent");
}

template <typename real>
void OperatorT<real>::degrid_slots(const void *grid, void *caller_vis) {
  if (wmode_) {
    WArgs<real> w;
    w.grid = grid;
    w.tasks = tasks_.as<Task>();
    w.order = task_order_.as<int32_t>();
    w.code = wcode_.as<int32_t>();
    w.factor = wfactor_.as<int64_t>();
    w.factors = wfactors_.get();
    w.weight = weight_.get();
    w.slot_out = ws_->slots;
    w.chunks = wchunks_.as<WChunk>();
    w.task_chunk = wtask_chunk_.as<int32_t>();
    w.chunk_values = wchunk_values_;
    w.Nu = Nu_;
    w.Nv = Nv_;
    w.Smax = fold_J_;
    mark_begin(kDegrid);
    cuda_check(launch_wdegrid<real>(w, ntasks_, win_rows_, win_cols_, ws_->stream),
               "w degrid");
    mark_end(kDegrid);
    return;
  }
  ApplyArgs<real> a;
  a.grid = grid;
  a.tasks = tasks_.as<Task>();
  a.batches = batches_.as<int2>();
  a.lane_code = lane_code_.as<int32_t>();
  a.frac = frac_.get();
  a.slot_out = caller_vis ? caller_vis : ws_->slots;
  a.slot_user = caller_vis ? slot_user_.as<int32_t>() : nullptr;
  a.keep_in = (caller_vis && keep_store_ && keep_vis_l2_ && ws_ == &own_) ? 1 : 0;
  a.Nu = Nu_;
  a.Nv = Nv_;
  a.win_stride = win_stride_;
  a.group_cells = group_;
  a.order = task_order_.as<int32_t>();
  mark_begin(kDegrid);
  cuda_check(launch_degrid<real>(a, poly_, J_, ntasks_, win_rows_, win_cols_, shape_, ws_->stream),
             "degrid");
  if (split_weights_) {
    if (caller_vis)
      cuda_check(launch_cmul<real>(caller_vis, wcaller_.get(), M_, false, ws_->stream), "weights");
    else
      cuda_check(launch_cmul<real>(ws_->slots, weight_.get(), S_, false, ws_->stream), "weights");
  }
  mark_end(kDegrid);
}

template <typename real>
void OperatorT<real>::grid_slots(void *grid, const void *caller_vis) {
  grid_core(grid, caller_vis ? caller_vis : ws_->slots,
            caller_vis ? slot_user_.as<int32_t>() : nullptr, ws_->tilebuf);
}

// G^H from visibilities in slot order (or caller order through slot_user)
// into `grid`, accumulating in the task windows at `windows`.
template <typename real>
void OperatorT<real>::grid_core(void *grid, const void *vis, const int32_t *slot_user,
                                void *windows) {
  if (wmode_) {
    WArgs<real> w;
    w.tilebuf = windows;
    w.tasks = tasks_.as<Task>();
    w.order = task_order_.as<int32_t>();
    w.code = wcode_.as<int32_t>();
    w.factor = wfactor_.as<int64_t>();
    w.factors = wfactors_.get();
    w.weight = weight_.get();
    w.slot_in = vis;
    w.chunks = wchunks_.as<WChunk>();
    w.task_chunk = wtask_chunk_.as<int32_t>();
    w.chunk_values = wchunk_values_;
    w.Nu = Nu_;
    w.Nv = Nv_;
    w.Smax = fold_J_;
    w.slot_stride = slot_stride_;
    mark_begin(kGrid);
    cuda_check(launch_wgrid<real>(w, ntasks_, win_rows_, win_cols_, ws_->stream),
               "w grid");
    mark_end(kGrid);
    fold_into(grid, windows, tile_tasks_.as<int32_t>());
    return;
  }
  ApplyArgs<real> a;
  a.tilebuf = windows;
  a.tasks = tasks_.as<Task>();
  a.batches = batches_.as<int2>();
  a.lane_code = lane_code_.as<int32_t>();
  a.frac = frac_.get();
  a.slot_in = vis;
  a.slot_user = slot_user;
  // reading caller order on the operator's own scratch: keep the vector in
  // L2 for the next forward's scattered stores (see kKeepVisL2Bytes)
  a.keep_in = (slot_user && keep_vis_l2_ && ws_ == &own_) ? 1 : 0;
  a.Nu = Nu_;
  a.Nv = Nv_;
  a.win_stride = win_stride_;
  a.group_cells = group_;
  a.order = task_order_.as<int32_t>();
  a.slot_stride = slot_stride_;
  mark_begin(kGrid);
  cuda_check(launch_grid<real>(a, poly_, J_, ntasks_, win_rows_, win_cols_, shape_, ws_->stream),
             "grid");
  mark_end(kGrid);
  fold_into(grid, windows, tile_tasks_.as<int32_t>());
}

template <typename real>
void OperatorT<real>::walk_grid(void *grid) {
  WalkArgs<real> a;
  a.tasks = walk_tasks_.as<Task>();
  a.order = walk_order_.as<int32_t>();
  a.counts = walk_counts_.as<int32_t>();
  a.colstart = walk_colstart_.as<int32_t>();
  a.frac = walk_frac_.get();
  a.slot_in = ws_->slots;
  a.tilebuf = ws_->tilebuf;
  a.slot_stride = slot_stride_;
  a.win_stride = walk_win_stride_;
  a.win_rows = walk_win_rows_;
  a.max_steps = walk_max_steps_;
  mark_begin(kGrid);
  cuda_check(launch_walk_grid<real>(a, poly_, J_, walk_ntasks_, kWalkThreads, ws_->stream),
             "walk grid");
  mark_end(kGrid);
  fold_into(grid, ws_->tilebuf, walk_tile_tasks_.as<int32_t>());
}

template <typename real>
void OperatorT<real>::fold_into(void *grid, const void *windows, const int32_t *tile_tasks) {
  FoldArgs f;
  f.tilebuf = windows;
  f.slot_stride = slot_stride_;
  f.tile_tasks = tile_tasks;
  f.tu_start = tu_start_.as<int32_t>();
  f.tv_start = tv_start_.as<int32_t>();
  f.tu_of = tu_of_.as<int32_t>();
  f.tv_of = tv_of_.as<int32_t>();
  f.ntu = ntu_;
  f.ntv = ntv_;
  f.Ju = fold_J_;
  f.Jv = fold_Jv_;
  f.Nu = Nu_;
  f.Nv = Nv_;
  f.grid = grid;
  mark_begin(kFold);
  cuda_check(launch_fold<real>(f, ws_->stream), "fold");
  mark_end(kFold);
}

template <typename real>
void OperatorT<real>::degrid_on_stream(const void *grid, void *y) {
  if (fused_forward_) {
    degrid_slots(grid, y);
    return;
  }
  degrid_slots(grid);
  mark_begin(kCompact);
  cuda_check(launch_compact<real>(ws_->slots, user_slot_.as<int32_t>(), y, M_, ws_->stream),
             "compact");
  mark_end(kCompact);
}

template <typename real>
void OperatorT<real>::grid_on_stream(const void *y, void *grid) {
  if (fused_adjoint_) {
    grid_slots(grid, y);
    return;
  }
  mark_begin(kExpand);
  cuda_check(launch_expand<real>(y, slot_user_.as<int32_t>(), ws_->slots, S_, ws_->stream,
                                 keep_vis_l2_ && ws_ == &own_, slot_weights()),
             "expand");
  mark_end(kExpand);
  grid_slots(grid);
}

template <typename real>
FftArgs OperatorT<real>::fft_args() const {
  FftArgs f;
  f.Nx = Nx_;
  f.Ny = Ny_;
  f.Nu = Nu_;
  f.Nv = Nv_;
  f.x0 = x0_;
  f.y0 = y0_;
  f.su = reinterpret_cast<const float *>(su_active());
  f.sv = reinterpret_cast<const float *>(sv_d_.get());
  f.tw_u = tw_u_.get();
  return f;
}

template <typename real>
FftColArgs OperatorT<real>::col_args(const void *in, void *out) const {
  FftColArgs c;
  c.in = in;
  c.out = out;
  c.Nv = Nv_;
  c.W = Nu_;
  c.ld = Nu_;
  c.y0 = y0_;
  c.Ny = Ny_;
  c.tw_v = tw_v_.get();
  return c;
}

template <typename real>
void OperatorT<real>::forward_grid(const void *x) {
  if (use_fused_fft()) {
    // row transforms of the image rows into ws->pad (its other rows stay
    // zero), then the column transform into ws->work
    mark_begin(kFftF);
    cuda_check(launch_fft_rows_forward(fft_args(), x, ws_->pad, ws_->stream), "fft rows");
    if (own_cols_)
      cuda_check(launch_fft_cols(false, col_args(ws_->pad, ws_->work), ws_->stream), "fft columns");
    else
      cufft_check(Traits<real>::exec(ws_->fft_cols, ws_->pad, ws_->work, CUFFT_FORWARD),
                  "cufftExec");
    mark_end(kFftF);
    return;
  }
  mark_begin(kPad);
  cuda_check(launch_pad<real>(x, su_active(), sv_d_.as<real>(), ws_->pad, Nx_, Ny_, Nu_,
                              x0_, y0_, ws_->stream),
             "pad");
  mark_end(kPad);
  mark_begin(kFftF);
  cufft_check(Traits<real>::exec(ws_->fft, ws_->pad, ws_->work, CUFFT_FORWARD), "cufftExec");
  mark_end(kFftF);
}

template <typename real>
void OperatorT<real>::inverse_grid(void *x) {
  if (use_fused_fft()) {
    mark_begin(kFftI);
    if (own_cols_)
      cuda_check(launch_fft_cols(true, col_args(ws_->work, ws_->work), ws_->stream), "fft columns");
    else
      cufft_check(Traits<real>::exec(ws_->fft_cols, ws_->work, ws_->work, CUFFT_INVERSE),
                  "cufftExec");
    cuda_check(launch_fft_rows_inverse(fft_args(), ws_->work, x, ws_->stream), "fft rows");
    mark_end(kFftI);
    return;
  }
  mark_begin(kFftI);
  cufft_check(Traits<real>::exec(ws_->fft, ws_->work, ws_->work, CUFFT_INVERSE), "cufftExec");
  mark_end(kFftI);
  mark_begin(kCrop);
  cuda_check(launch_crop<real>(ws_->work, su_active(), sv_d_.as<real>(), x, Nx_, Ny_, Nu_,
                               x0_, y0_, ws_->stream),
             "crop");
  mark_end(kCrop);
}

template <typename real>
void OperatorT<real>::forward_slots(const void *x, void *caller_vis) {
  forward_grid(x);
  degrid_slots(ws_->work, caller_vis);
}

template <typename real>
void OperatorT<real>::adjoint_slots(void *x, const void *caller_vis, bool walk) {
  if (walk)
    walk_grid(ws_->work);
  else
    grid_slots(ws_->work, caller_vis);
  inverse_grid(x);
}

template <typename real>
void OperatorT<real>::normal_slots(const void *x, void *out) {
  if (one_pass_normal_) {
    // F Z S, then G^H G in one pass over each task into the task windows,
    // fold, and S^H Z^H F^H
    forward_grid(x);
    ApplyArgs<real> a;
    a.grid = ws_->work;
    a.tilebuf = ws_->tilebuf;
    a.tasks = tasks_.as<Task>();
    a.batches = batches_.as<int2>();
    a.lane_code = lane_code_.as<int32_t>();
    a.frac = frac_.get();
    a.Nu = Nu_;
    a.Nv = Nv_;
    a.win_stride = win_stride_;
    a.group_cells = group_;
    a.order = task_order_.as<int32_t>();
    a.slot_stride = slot_stride_;
    mark_begin(kGrid);
    cuda_check(launch_normal<real>(a, poly_, J_, ntasks_, win_rows_, win_cols_, kNormalShape,
                                   ws_->stream),
               "normal");
    mark_end(kGrid);
    fold_into(ws_->work, ws_->tilebuf, tile_tasks_.as<int32_t>());
    inverse_grid(out);
    return;
  }
  forward_slots(x);
  if (split_weights_)
    cuda_check(launch_cmul<real>(ws_->slots, weight_.get(), S_, true, ws_->stream), "weights");
  adjoint_slots(out);
}

template <typename real>
void OperatorT<real>::forward_on_stream(const void *x, void *y) {
  if (fused_forward_) {
    forward_slots(x, y);
    return;
  }
  forward_slots(x);
  mark_begin(kCompact);
  cuda_check(launch_compact<real>(ws_->slots, user_slot_.as<int32_t>(), y, M_, ws_->stream),
             "compact");
  mark_end(kCompact);
}

template <typename real>
void OperatorT<real>::adjoint_on_stream(const void *y, void *x) {
  // The grid kernel gathers caller order itself (fused_adjoint_), on the
  // operator's own scratch and on the request server's workspaces alike.
  if (fused_adjoint_) {
    adjoint_slots(x, y);
    return;
  }
  mark_begin(kExpand);
  if (walk_)
    cuda_check(launch_expand<real>(y, walk_user_.as<int32_t>(), ws_->slots, M_, ws_->stream,
                                   keep_vis_l2_ && ws_ == &own_,
                                   split_weights_ ? walk_weight_.get() : nullptr),
               "expand");
  else
    cuda_check(launch_expand<real>(y, slot_user_.as<int32_t>(), ws_->slots, S_, ws_->stream,
                                   keep_vis_l2_ && ws_ == &own_, slot_weights()),
               "expand");
  mark_end(kExpand);
  adjoint_slots(x, nullptr, walk_);
}

template <typename real>
WorkspaceSizes OperatorT<real>::workspace_sizes() const {
  WorkspaceSizes w;
  w.pad = int64_t(sizeof(C)) * Nu_ * Nv_;
  w.work = w.pad;
  w.tilebuf = int64_t(sizeof(C)) * slot_stride_ * std::max(ntasks_, 1);
  w.slots = int64_t(sizeof(C)) * std::max<int64_t>(S_, 1);
  return w;
}

// Enqueues f's launches on ws.stream with ws's scratch.  The coverage state
// is only read, so applies on different workspaces may run concurrently.
template <typename real>
void OperatorT<real>::with_workspace(const Workspace &ws, const std::function<void()> &f) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  ws_ = &ws;
  try {
    f();
  } catch (...) {
    ws_ = &own_;
    throw;
  }
  ws_ = &own_;
}

template <typename real>
void OperatorT<real>::forward_ws(const void *x, void *y, const Workspace &ws) {
  with_workspace(ws, [&] { forward_on_stream(x, y); });
}
template <typename real>
void OperatorT<real>::adjoint_ws(const void *y, void *x, const Workspace &ws) {
  with_workspace(ws, [&] { adjoint_on_stream(y, x); });
}

// The power iteration of power_method() with the normalisation done on the
// device: after round i, sq[i] = ||x||^2 (FP64, same reduction) and x is
// scaled by real(1 / sqrt(sq[i])), the host's arithmetic, so the estimates
// sqrt(sq[i]) are those of power_method() bit for bit.  The stopping rule is
// applied by the caller to the recorded estimates.
template <typename real>
void OperatorT<real>::power_ws(void *x, int first, int count, double *sq, double *partial,
                               const Workspace &ws) {
  Workspace w = ws;
  w.unit_norm = true;
  with_workspace(w, [&] {
    if (first == 0)
      cuda_check(launch_fill<real>(x, N_, 1.0 / std::sqrt(double(N_)), w.stream), "fill");
    for (int i = first; i < first + count; ++i) {
      normal_slots(x, x);
      cuda_check(launch_sq_norm<real>(x, N_, partial, sq + i, w.stream), "norm");
      cuda_check(launch_scale_rsqrt<real>(x, N_, sq + i, w.stream), "scale");
    }
  });
}

template <typename real>
void OperatorT<real>::normal(const void *x, void *out, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  run_recorded(3, x, out, [&] {
    normal_slots(x, out);
  });
  release(user);
}

template <typename real>
void OperatorT<real>::degrid(const void *grid, void *vis, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  degrid_on_stream(grid, vis);
  release(user);
}
template <typename real>
void OperatorT<real>::grid(const void *vis, void *grid, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  grid_on_stream(vis, grid);
  release(user);
}

// Scratch layout in the fixed array: the task windows, then (when the grid
// kernel does not gather caller order itself) the slot buffer, each starting
// on a 256-byte boundary.
template <typename real>
int64_t OperatorT<real>::no_alloc_bytes() const {
  auto up = [](int64_t b) { return (b + 255) / 256 * 256; };
  return up(int64_t(sizeof(C)) * slot_stride_ * std::max(ntasks_, 1)) +
         (fused_adjoint_ ? 0 : up(int64_t(sizeof(C)) * std::max<int64_t>(S_, 1)));
}

template <typename real>
void OperatorT<real>::grid_no_alloc(const void *vis, void *grid, cudaStream_t user) {
  DeviceGuard guard(device_);
  const int64_t need = no_alloc_bytes();
  if (need > int64_t(static_scratch_bytes()))
    throw Error(kInvalidArgument,
                "purify_gb300_grid_no_alloc: this operator needs " + std::to_string(need) +
                    " bytes of scratch, the fixed array holds " +
                    std::to_string(static_scratch_bytes()));
  void *scratch = nullptr;
  cuda_check(static_scratch_address(&scratch), "cudaGetSymbolAddress");
  unsigned char *base = static_cast<unsigned char *>(scratch);
  void *windows = base;
  void *slots = base + (int64_t(sizeof(C)) * slot_stride_ * std::max(ntasks_, 1) + 255) / 256 * 256;
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  // expand writes every slot (0 for null slots) and the grid kernels write
  // every cell of every task window, so nothing left in the array from an
  // earlier call is read.
  if (fused_adjoint_) {
    grid_core(grid, vis, slot_user_.as<int32_t>(), windows);
  } else {
    cuda_check(launch_expand<real>(vis, slot_user_.as<int32_t>(), slots, S_, stream_, false,
                                   slot_weights()),
               "expand");
    grid_core(grid, slots, nullptr, windows);
  }
  release(user);
}

// Applies on the operator's own scratch are recorded into a CUDA graph the
// second time they are made with the same buffers and replayed from then on:
// the chain's launches are then one graph launch.  The graph holds the
// buffer addresses only; everything else it reads (coverage state, the
// correction and norm) is read from device memory when it runs.
template <typename real>
void OperatorT<real>::run_recorded(int kind, const void *in, void *out,
                                   const std::function<void()> &enqueue) {
  if (timing_ || ws_ != &own_) {
    enqueue();
    return;
  }
  const GraphKey key{kind, in, out};
  auto it = graphs_.find(key);
  if (it != graphs_.end()) {
    cuda_check(cudaGraphLaunch(it->second, stream_), "cudaGraphLaunch");
    return;
  }
  if (!seen_.count(key)) {
    seen_.insert(key);
    if (seen_.size() > 64) seen_.clear();
    enqueue();
    return;
  }
  if (graphs_.size() >= 16) drop_graphs();
  cudaGraph_t g = nullptr;
  cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture");
  try {
    enqueue();
  } catch (...) {
    cudaStreamEndCapture(stream_, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  cuda_check(cudaStreamEndCapture(stream_, &g), "capture");
  cudaGraphExec_t e = nullptr;
  const cudaError_t r = cudaGraphInstantiate(&e, g, 0);
  cudaGraphDestroy(g);
  cuda_check(r, "cudaGraphInstantiate");
  graphs_[key] = e;
  cuda_check(cudaGraphLaunch(e, stream_), "cudaGraphLaunch");
}

template <typename real>
void OperatorT<real>::drop_graphs() {
  for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

template <typename real>
void OperatorT<real>::forward(const void *x, void *y, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  run_recorded(1, x, y, [&] { forward_on_stream(x, y); });
  release(user);
}
template <typename real>
void OperatorT<real>::adjoint(const void *y, void *x, cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  join(user);
  run_recorded(2, y, x, [&] { adjoint_on_stream(y, x); });
  release(user);
}

template <typename real>
void OperatorT<real>::ensure_host_staging() {
  if (staging_) return;
  int64_t *cnt = &info_.device_bytes;
  x128_.alloc(16 * size_t(N_), cnt);
  y128_.alloc(16 * size_t(M_), cnt);
  if (sizeof(real) != sizeof(double)) {
    xc_.alloc(sizeof(C) * size_t(N_), cnt);
    yc_.alloc(sizeof(C) * size_t(M_), cnt);
    cuda_check(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
    copy_ev_.resize(kCopyChunks + 1);
    for (cudaEvent_t &e : copy_ev_)
      cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
  }
  staging_ = true;
}

template <typename real>
void OperatorT<real>::upload_c128(const double *host, void *stage, void *dev, int64_t n) {
  const int64_t chunk = std::max<int64_t>(kCopyChunkMin, (n + kCopyChunks - 1) / kCopyChunks);
  // the staging buffer is free once the work before this call on stream_ is
  cuda_check(cudaEventRecord(copy_ev_[kCopyChunks], stream_), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(copy_stream_, copy_ev_[kCopyChunks], 0), "cudaStreamWaitEvent");
  for (int64_t off = 0, k = 0; off < n; off += chunk, ++k) {
    const int64_t len = std::min(chunk, n - off);
    char *st = static_cast<char *>(stage) + 16 * off;
    cuda_check(cudaMemcpyAsync(st, host + 2 * off, 16 * size_t(len), cudaMemcpyHostToDevice,
                               copy_stream_),
               "H2D");
    cuda_check(cudaEventRecord(copy_ev_[k], copy_stream_), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(stream_, copy_ev_[k], 0), "cudaStreamWaitEvent");
    cuda_check(launch_from_c128<real>(st, static_cast<C *>(dev) + off, len, stream_), "convert");
  }
}

template <typename real>
void OperatorT<real>::download_c128(const void *dev, void *stage, double *host, int64_t n) {
  const int64_t chunk = std::max<int64_t>(kCopyChunkMin, (n + kCopyChunks - 1) / kCopyChunks);
  for (int64_t off = 0, k = 0; off < n; off += chunk, ++k) {
    const int64_t len = std::min(chunk, n - off);
    char *st = static_cast<char *>(stage) + 16 * off;
    cuda_check(launch_to_c128<real>(static_cast<const C *>(dev) + off, st, len, stream_),
               "convert");
    cuda_check(cudaEventRecord(copy_ev_[k], stream_), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(copy_stream_, copy_ev_[k], 0), "cudaStreamWaitEvent");
    cuda_check(cudaMemcpyAsync(host + 2 * off, st, 16 * size_t(len), cudaMemcpyDeviceToHost,
                               copy_stream_),
               "D2H");
  }
  // later work on stream_ (which may rewrite the staging buffer) follows the copies
  cuda_check(cudaEventRecord(copy_ev_[kCopyChunks], copy_stream_), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(stream_, copy_ev_[kCopyChunks], 0), "cudaStreamWaitEvent");
}

template <typename real>
void OperatorT<real>::forward_host(const double *x, double *y) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  ensure_host_staging();
  if (sizeof(real) != sizeof(double)) {
    upload_c128(x, x128_.get(), xc_.get(), N_);
    forward_on_stream(xc_.get(), yc_.get());
    download_c128(yc_.get(), y128_.get(), y, M_);
    cuda_check(cudaStreamSynchronize(stream_), "forward_host");
    return;
  }
  cuda_check(cudaMemcpyAsync(x128_.get(), x, 16 * size_t(N_), cudaMemcpyHostToDevice, stream_),
             "H2D");
  forward_on_stream(x128_.get(), y128_.get());
  cuda_check(cudaMemcpyAsync(y, y128_.get(), 16 * size_t(M_), cudaMemcpyDeviceToHost, stream_),
             "D2H");
  cuda_check(cudaStreamSynchronize(stream_), "forward_host");
}

template <typename real>
void OperatorT<real>::adjoint_host(const double *y, double *x) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  ensure_host_staging();
  if (sizeof(real) != sizeof(double)) {
    upload_c128(y, y128_.get(), yc_.get(), M_);
    adjoint_on_stream(yc_.get(), xc_.get());
    download_c128(xc_.get(), x128_.get(), x, N_);
    cuda_check(cudaStreamSynchronize(stream_), "adjoint_host");
    return;
  }
  cuda_check(cudaMemcpyAsync(y128_.get(), y, 16 * size_t(M_), cudaMemcpyHostToDevice, stream_),
             "H2D");
  adjoint_on_stream(y128_.get(), x128_.get());
  cuda_check(cudaMemcpyAsync(x, x128_.get(), 16 * size_t(N_), cudaMemcpyDeviceToHost, stream_),
             "D2H");
  cuda_check(cudaStreamSynchronize(stream_), "adjoint_host");
}

// Power iteration on Phi'^H Phi' from the normalised all-ones vector
// (operators.h:390-391).  The eigenvalue estimate is the FP64 2-norm of the
// iterate after each round; the iteration stops when its relative change
// drops below tol^2, and ||Phi'|| = sqrt(estimate).  The reductions are FP64
// and deterministic.
template <typename real>
double OperatorT<real>::power_method(int iters, double tol) {
  DeviceGuard guard(device_);
  if (iters <= 0) {
    set_norm(1.0);
    return 1.0;
  }
  double result = 0;
  {
    std::lock_guard<std::mutex> lock(mu_);
    if (!pm_ready_) {
      int64_t *cnt = &info_.device_bytes;
      pm_x_.alloc(sizeof(C) * size_t(N_), cnt);
      pm_ready_ = true;
    }
    const double saved = norm_;
    norm_ = 1.0;
    upload_correction();
    try {
      cuda_check(launch_fill<real>(pm_x_.get(), N_, 1.0 / std::sqrt(double(N_)), stream_), "fill");
      double old_value = 0;
      for (int i = 0; i < iters; ++i) {
        // visibilities stay in slot order between the two halves
        normal_slots(pm_x_.get(), pm_x_.get());
        cuda_check(launch_sq_norm<real>(pm_x_.get(), N_, norm_partial_.as<double>(),
                                        norm_out_.as<double>(), stream_),
                   "norm");
        double sq = 0;
        cuda_check(cudaMemcpyAsync(&sq, norm_out_.get(), sizeof(double), cudaMemcpyDeviceToHost,
                                   stream_),
                   "D2H");
        cuda_check(cudaStreamSynchronize(stream_), "power_method");
        const double value = std::sqrt(sq);
        if (!(value > 0)) throw Error(kNormNotPositive, "Operator norm is not greater than zero.");
        cuda_check(launch_scale<real>(pm_x_.get(), N_, 1.0 / value, stream_), "scale");
        if (tol * tol > std::abs(old_value - value) / old_value) {
          old_value = value;
          break;
        }
        old_value = value;
      }
      result = std::sqrt(old_value);
    } catch (...) {
      norm_ = saved;
      upload_correction();
      throw;
    }
  }
  set_norm(result);
  return result;
}

template <typename real>
void OperatorT<real>::mark_begin(int stage) {
  if (!timing_) return;
  if (marks_used_ == marks_.size()) {
    if (marks_.size() >= 4096) {
      drain_timing();
    } else {
      Mark m{stage, nullptr, nullptr};
      cuda_check(cudaEventCreate(&m.a), "cudaEventCreate");
      cuda_check(cudaEventCreate(&m.b), "cudaEventCreate");
      event_pool_.push_back(m.a);
      event_pool_.push_back(m.b);
      marks_.push_back(m);
    }
  }
  marks_[marks_used_].stage = stage;
  cuda_check(cudaEventRecord(marks_[marks_used_].a, ws_->stream), "cudaEventRecord");
}
template <typename real>
void OperatorT<real>::mark_end(int) {
  if (!timing_) return;
  cuda_check(cudaEventRecord(marks_[marks_used_].b, ws_->stream), "cudaEventRecord");
  ++marks_used_;
}
template <typename real>
void OperatorT<real>::drain_timing() {
  cuda_check(cudaStreamSynchronize(stream_), "timing");
  for (size_t k = 0; k < marks_used_; ++k) {
    float ms = 0;
    cuda_check(cudaEventElapsedTime(&ms, marks_[k].a, marks_[k].b), "cudaEventElapsedTime");
    stage_ms_[marks_[k].stage] += ms;
    stage_n_[marks_[k].stage] += 1;
  }
  marks_used_ = 0;
}
template <typename real>
void OperatorT<real>::set_stage_timing(bool on) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  if (on) {
    drain_timing();
    for (int k = 0; k < kStages; ++k) {
      stage_ms_[k] = 0;
      stage_n_[k] = 0;
    }
  }
  timing_ = on;
}
template <typename real>
void OperatorT<real>::stage_times(double *total_ms, int64_t *launches) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  drain_timing();
  for (int k = 0; k < kStages; ++k) {
    if (total_ms) total_ms[k] = stage_ms_[k];
    if (launches) launches[k] = stage_n_[k];
  }
}

}  // namespace

void correction_factors(int kernel, int Ju, int Jv, int imsizey, int imsizex, double os,
                        double *S) {
  const int Nu = int(std::floor(imsizex * os)), Nv = int(std::floor(imsizey * os));
  const int x0 = int(std::floor(Nu * 0.5 - imsizex * 0.5));
  const int y0 = int(std::floor(Nv * 0.5 - imsizey * 0.5));
  const GriddingKernel ku(kernel, Ju, os), kv(kernel, Jv, os);
  std::vector<double> su(imsizex);
  for (int i = 0; i < imsizex; ++i) su[i] = 1.0 / ku.correction((x0 + i + 0.5) / Nu - 0.5);
  for (int j = 0; j < imsizey; ++j) {
    const double a = 1.0 / kv.correction((y0 + j + 0.5) / Nv - 0.5);
    for (int i = 0; i < imsizex; ++i) S[size_t(j) * imsizex + i] = a * su[i];
  }
}

std::unique_ptr<Operator> Operator::create(const OperatorConfig &cfg) {
  if (cfg.imsizex <= 0 || cfg.imsizey <= 0) throw Error(kInvalidArgument, "empty image");
  // The zero-padding operator places the image inside the grid
  // (operators.h:147-183), which needs a grid at least as large as the image.
  if (!(cfg.oversample_ratio >= 1.0))
    throw Error(kInvalidArgument, "oversample_ratio must be >= 1");
  if (cfg.M < 0) throw Error(kInvalidArgument, "negative number of visibilities");
  if (cfg.M > 0 && (!cfg.u || !cfg.v)) throw Error(kInvalidArgument, "u and v must be given");
  const std::string why = check_kernel_request(cfg.kernel, cfg.Ju, cfg.Jv);
  if (!why.empty()) throw Error(kInvalidArgument, why);
  if (cfg.Ju < 1 || cfg.Jv < 1) throw Error(kInvalidArgument, "kernel support must be >= 1");
  if (cfg.Ju != cfg.Jv && (cfg.kernel == kKB || cfg.kernel == kKBMin))
    throw Error(kInvalidArgument,
                "Ju != Jv with a Kaiser-Bessel kernel: the reference builds G with the Jv kernel "
                "on the u axis and the Ju kernel on the v axis (operators.h:322-324), so one "
                "axis is evaluated outside its support, where the kernel is not a number");
  if (cfg.Ju != cfg.Jv && cfg.w_term)
    throw Error(kUnsupported, "w-projection with Ju != Jv (non-square rows) is not supported");
  if (!cfg.w_term && std::max(cfg.Ju, cfg.Jv) > kMaxWSupport)
    throw Error(kUnsupported, "kernel support must be between 1 and 32 taps");
  if (cfg.w_term && cfg.Ju > kMaxWSupport)
    throw Error(kUnsupported, "kernel support must be between 1 and 32 taps");
  if (cfg.class_cap < 0 || cfg.class_cap > 16)
    throw Error(kInvalidArgument, "class_cap must be 0 (default) or in [1, 16]");
  if (cfg.cell_group < 0 || cfg.cell_group > 3)
    throw Error(kInvalidArgument, "cell_group must be 0 (automatic), 1, 2 or 3");
  if (cfg.cell_group >= 2 && (cfg.fp64 || cfg.Ju > kMaxGroupJ || cfg.w_term || cfg.Ju != cfg.Jv))
    throw Error(kUnsupported,
                "2 x 2 and row-pair work items need complex<float>, J <= 6 and no w-projection");
  if (cfg.w_term && (cfg.M > 0 && !cfg.w))
    throw Error(kInvalidArgument, "w-projection needs the w coordinates");
  if (cfg.w_term && (cfg.Jw < 1 || cfg.Jw + cfg.Ju - 1 > kMaxWSupport) && !cfg.jw_rows)
    throw Error(kUnsupported, "w-projection support Jw + J - 1 must be between 1 and 32");
  if (cfg.threads != 0 && (cfg.threads % 32 != 0 || cfg.threads < 32 || cfg.threads > 256))
    throw Error(kInvalidArgument, "threads must be a multiple of 32 in [32, 256]");
  if (cfg.fp64) return std::unique_ptr<Operator>(new OperatorT<double>(cfg));
  return std::unique_ptr<Operator>(new OperatorT<float>(cfg));
}

}  // namespace pg
