#include "batch.h"
#include "operator.h"

#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <type_traits>
#include <utility>
#include <vector>

#include "device_kernels.h"
#include "device_util.h"
#include "fft_kernels.h"
#include "gridding_kernels.h"
#include "plan.h"

namespace pg {
namespace {

size_t up256(size_t b) { return (std::max<size_t>(b, 1) + 255) / 256 * 256; }

// Sub-allocations of one device allocation: offsets are reserved first, the
// allocation is made once, then each array is at base + offset.
class Arena {
 public:
  size_t reserve(size_t bytes) {
    const size_t off = total_;
    total_ += up256(bytes);
    return off;
  }
  void allocate(int64_t *counter) { buf_.alloc(total_, counter); }
  template <typename T>
  T *at(size_t off) const {
    return reinterpret_cast<T *>(static_cast<char *>(buf_.get()) + off);
  }

 private:
  size_t total_ = 0;
  DeviceBuffer buf_;
};

// Graph modes: which stages one replay runs.
enum Mode { kForward = 1, kAdjoint = 2, kBoth = 3, kPower = 7, kDegridOnly = 8, kGridOnly = 16 };

template <typename real>
class BatchT final : public Batch {
 public:
  explicit BatchT(const BatchConfig &cfg);
  ~BatchT() override;
  void bind(const void *const *x_in, void *const *vis, void *const *x_out,
            cudaStream_t stream) override;
  void apply(int directions, cudaStream_t stream) override;
  void set_norms(const double *norms) override;
  void power_method(int iters, double tol, double *norms) override;
  void get_norms(double *norms) const override;
  BatchInfo info() const override { return info_; }
  void set_launch_shapes(int degrid_threads, int grid_threads) override;
  double time_apply(int directions, int reps) override;

 private:
  using C = std::complex<real>;
  struct Chan {
    int Nx = 0, Ny = 0, Nu = 0, Nv = 0, x0 = 0, y0 = 0;
    int64_t M = 0, S = 0, slot_stride = 0;
    int ntasks = 0, ntu = 0, ntv = 0, win_rows = 0, win_cols = 0, win_stride = 0;
    int group = 0, in_group = 0;
    bool unit = true;
    double norm = 1.0;
    std::vector<double> su, sv;  // 1 / ft kernel at the image pixels (unscaled)
    Arena mem;                   // coverage state and scratch of this channel
    size_t o_frac = 0, o_weight = 0, o_slot_user = 0, o_user_slot = 0, o_batches = 0,
           o_lane = 0, o_tile_tasks = 0, o_tu_start = 0, o_tv_start = 0, o_tu_of = 0,
           o_tv_of = 0, o_su = 0, o_sv = 0, o_tilebuf = 0, o_slots = 0, o_pm_x = 0, o_pm_vis = 0,
           o_wvis = 0;
  };
  // Channels of one grid size.  FP32 groups of a power-of-two width are
  // "fused": their grids are interleaved by rows (row r of the group holds
  // row r of every member, member k at columns k Nu ..., row stride
  // ld = members x Nu), the padding and the row FFTs of all members run as
  // one row-pass launch, and one column pass (launch_fft_cols; a strided
  // cuFFT plan where that does not apply) transforms every member's columns.
  // The other groups keep contiguous grids (ld = Nu), a batched 2-D plan and
  // the grouped pad / crop kernels.
  struct SizeGroup {
    int Nu = 0, Nv = 0;
    std::vector<int> chans;
    size_t o_pad = 0, o_work = 0;
    cufftHandle fft = 0;  // fused: the cuFFT column plan (if any); else the batched 2-D plan
    bool fft_ok = false;
    bool fused = false, own_cols = false;
    int ld = 0, max_ny = 0;
    // fused: member channel indices, row and column twiddles
    size_t o_members = 0, o_tw = 0, o_twv = 0;
  };
  FftColArgs col_args(const SizeGroup &g, bool inverse) const;
  void upload_corrections();
  void upload_tables(cudaStream_t s);
  void record(int mode);
  cudaGraphExec_t graph_for(int mode);
  void drop_graphs();
  // Binds every channel to its own image and visibility buffers (power method
  // and timing); the caller restores the user's binding.
  void bind_internal();
  void join(cudaStream_t user);
  void release(cudaStream_t user);
  // a channel's grids inside its group's buffers
  size_t grid_offset(int c) const {
    const SizeGroup &g = groups_[chans_[c].group];
    return size_t(chans_[c].in_group) * size_t(g.Nu) * (g.fused ? 1 : size_t(g.Nv));
  }
  void *pad_of(int c) const {
    return shared_.at<C>(groups_[chans_[c].group].o_pad) + grid_offset(c);
  }
  void *work_of(int c) const {
    return shared_.at<C>(groups_[chans_[c].group].o_work) + grid_offset(c);
  }

  int device_ = 0, J_ = 0, nch_ = 0;
  int cfg_group_ = 1;  // cells per work item along each axis (every channel's plan)
  PolyTable<real> poly_{};
  LaunchShape degrid_shape_, grid_shape_;
  std::unique_ptr<Chan[]> chans_;
  std::vector<SizeGroup> groups_;
  int ntasks_ = 0, win_rows_ = 0, win_cols_ = 0;
  Arena shared_;  // grouped task list, argument tables, padded and FFT grids
  size_t o_tasks_ = 0, o_task_base_ = 0, o_fwd_ = 0, o_adj_ = 0, o_folds_ = 0, o_io_ = 0,
         o_partial_ = 0, o_sq_ = 0, o_inv_ = 0, o_map_pix_ = 0, o_map_pad_ = 0, o_map_slot_ = 0,
         o_map_tile_ = 0,
         o_map_wvis_ = 0,
         o_order_ = 0;
  // block maps of the grouped element-wise launches: {channel, block}
  std::vector<int2> map_pix_, map_slot_, map_tile_;
  std::vector<int2> map_pad_;  // pixels of the channels of unfused size groups (pad / crop)
  std::vector<int2> map_wvis_;  // caller-ordered visibilities of the channels with weights
  std::vector<ApplyArgs<real>> fwd_, adj_;
  std::vector<FoldArgs> folds_;
  std::vector<ChannelIO<real>> io_;
  std::vector<const void *> bound_x_in_;
  std::vector<void *> bound_vis_, bound_x_out_;
  BatchInfo info_;

  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_in_ = nullptr, ev_out_ = nullptr;
  std::map<int, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs_;
  std::mutex mu_;
};

template <typename real>
BatchT<real>::BatchT(const BatchConfig &cfg) {
  device_ = cfg.device;
  DeviceGuard guard(device_);
  nch_ = int(cfg.channels.size());
  J_ = cfg.J;
  cfg_group_ = cfg.cell_group;
  degrid_shape_.threads = cfg.degrid_threads > 0 ? cfg.degrid_threads : cfg.threads;
  grid_shape_.threads = cfg.grid_threads > 0 ? cfg.grid_threads : cfg.threads;

  // One kernel fit serves every channel: it depends on the kernel, the
  // support and the oversampling only.
  const GriddingKernel kern(cfg.kernel, J_, cfg.oversample_ratio);
  const int nc = PolyCount<real>::value;
  const AxisFit fit = fit_axis(kern, J_, nc);
  std::memset(&poly_, 0, sizeof(poly_));
  for (int j = 0; j < J_; ++j)
    for (int s = 0; s < fit.nsub; ++s)
      for (int k = 0; k < nc; ++k) {
        const real c = real(fit.coef[(size_t(j) * fit.nsub + s) * nc + k]);
        poly_.u.c[j][s][k] = c;
        poly_.v.c[j][s][k] = c;
      }
  poly_.nsub_u = poly_.nsub_v = fit.nsub;

  cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_in_, cudaEventDisableTiming), "cudaEventCreate");
  cuda_check(cudaEventCreateWithFlags(&ev_out_, cudaEventDisableTiming), "cudaEventCreate");

  chans_.reset(new Chan[nch_]);
  std::vector<Task> tasks;
  std::vector<int32_t> order;  // launch order of the grouped tasks
  std::vector<int32_t> task_base(nch_);
  for (int c = 0; c < nch_; ++c) {
    const ChannelSpec &spec = cfg.channels[c];
    Chan &ch = chans_[c];
    ch.Nx = spec.imsizex;
    ch.Ny = spec.imsizey;
    ch.Nu = int(std::floor(spec.imsizex * cfg.oversample_ratio));
    ch.Nv = int(std::floor(spec.imsizey * cfg.oversample_ratio));
    ch.x0 = int(std::floor(ch.Nu * 0.5 - ch.Nx * 0.5));
    ch.y0 = int(std::floor(ch.Nv * 0.5 - ch.Ny * 0.5));
    ch.M = spec.M;
    ch.su.resize(ch.Nx);
    ch.sv.resize(ch.Ny);
    for (int i = 0; i < ch.Nx; ++i)
      ch.su[i] = 1.0 / kern.correction((ch.x0 + i + 0.5) / ch.Nu - 0.5);
    for (int j = 0; j < ch.Ny; ++j)
      ch.sv[j] = 1.0 / kern.correction((ch.y0 + j + 0.5) / ch.Nv - 0.5);
    task_base[c] = int32_t(tasks.size());
    // Coverage plan of this channel, uploaded into its own allocation.
    PlanRequest rq;
    rq.u = spec.u;
    rq.v = spec.v;
    rq.weights = spec.weights;
    rq.M = spec.M;
    rq.Nu = ch.Nu;
    rq.Nv = ch.Nv;
    rq.Ju = rq.Jv = J_;
    rq.tile = cfg.tile;
    rq.max_per_item = cfg.max_per_item;
    rq.group = cfg.cell_group;
    rq.warps = (cfg.grid_threads > 0 ? cfg.grid_threads : cfg.threads) / 32;
    Plan plan;
    try {
      plan = build_plan(rq);
    } catch (const std::invalid_argument &e) {
      throw Error(kInvalidArgument, "channel " + std::to_string(c) + ": " + e.what());
    }
    ch.S = plan.S;
    ch.unit = plan.unit_weights;
    ch.ntasks = int(plan.tasks.size());
    ch.ntu = plan.tu.n;
    ch.ntv = plan.tv.n;
    ch.win_rows = plan.win_rows;
    ch.win_cols = plan.win_cols;
    ch.win_stride = plan.win_stride;
    ch.slot_stride = int64_t(plan.win_rows) * plan.win_cols;
    for (Task tk : plan.tasks) {
      tk.channel = c;
      tasks.push_back(tk);
    }
    // each channel's own launch order, channels one after the other (the
    // tasks of one grid stay together, so its windows share L2)
    for (int32_t k : plan.task_order) order.push_back(task_base[c] + k);
    const size_t nb = plan.batch_base.size();
    Arena &m = ch.mem;
    ch.o_frac = m.reserve(sizeof(C) * ch.S);
    ch.o_weight = ch.unit ? 0 : m.reserve(sizeof(C) * ch.S);
    ch.o_wvis = ch.unit ? 0 : m.reserve(sizeof(C) * ch.M);
    ch.o_slot_user = m.reserve(sizeof(int32_t) * ch.S);
    ch.o_user_slot = m.reserve(sizeof(int32_t) * ch.M);
    ch.o_batches = m.reserve(sizeof(int2) * nb);
    ch.o_lane = m.reserve(sizeof(int32_t) * plan.lane_code.size());
    ch.o_tile_tasks = m.reserve(sizeof(int32_t) * plan.tile_tasks.size());
    ch.o_tu_start = m.reserve(sizeof(int32_t) * plan.tu.start.size());
    ch.o_tv_start = m.reserve(sizeof(int32_t) * plan.tv.start.size());
    ch.o_tu_of = m.reserve(sizeof(int32_t) * plan.tu.of.size());
    ch.o_tv_of = m.reserve(sizeof(int32_t) * plan.tv.of.size());
    ch.o_su = m.reserve(sizeof(real) * ch.Nx);
    ch.o_sv = m.reserve(sizeof(real) * ch.Ny);
    ch.o_tilebuf = m.reserve(sizeof(C) * size_t(ch.slot_stride) * std::max(ch.ntasks, 1));
    ch.o_slots = m.reserve(sizeof(C) * ch.S);
    ch.o_pm_x = m.reserve(sizeof(C) * size_t(ch.Nx) * ch.Ny);
    ch.o_pm_vis = m.reserve(sizeof(C) * ch.M);
    m.allocate(&info_.device_bytes);
    std::vector<C> fr(ch.S);
    for (int64_t i = 0; i < ch.S; ++i) {
      // the phase sign (-1)^(k_u + k_v) rides in the sign of t_u
      const real tu = fraction_in_cell<real>(plan.frac_u[i]);
      fr[i] = C(plan.flip[i] ? -tu : tu, fraction_in_cell<real>(plan.frac_v[i]));
    }
    auto put = [&](size_t off, const void *src, size_t bytes) {
      if (bytes)
        cuda_check(cudaMemcpyAsync(m.at<char>(off), src, bytes, cudaMemcpyHostToDevice, stream_),
                   "upload");
    };
    put(ch.o_frac, fr.data(), sizeof(C) * ch.S);
    std::vector<C> wt;
    std::vector<C> wv;
    if (!ch.unit) {
      // the weights themselves (the plan folds the phase sign into them; it
      // rides in t_u here), in slot order for G^H and caller order for G
      wt.resize(ch.S);
      for (int64_t i = 0; i < ch.S; ++i) {
        const std::complex<double> w = plan.flip[i] ? -plan.weight[i] : plan.weight[i];
        wt[i] = C(real(w.real()), real(w.imag()));
      }
      put(ch.o_weight, wt.data(), sizeof(C) * ch.S);
      wv.resize(ch.M);
      for (int64_t k = 0; k < ch.M; ++k)
        wv[k] = C(real(spec.weights[k].real()), real(spec.weights[k].imag()));
      put(ch.o_wvis, wv.data(), sizeof(C) * ch.M);
    }
    put(ch.o_slot_user, plan.slot_user.data(), sizeof(int32_t) * ch.S);
    put(ch.o_user_slot, plan.user_slot.data(), sizeof(int32_t) * ch.M);
    std::vector<int2> bt(nb);
    for (size_t k = 0; k < nb; ++k) bt[k] = int2{plan.batch_base[k], plan.batch_kmax[k]};
    put(ch.o_batches, bt.data(), sizeof(int2) * nb);
    put(ch.o_lane, plan.lane_code.data(), sizeof(int32_t) * plan.lane_code.size());
    put(ch.o_tile_tasks, plan.tile_tasks.data(), sizeof(int32_t) * plan.tile_tasks.size());
    put(ch.o_tu_start, plan.tu.start.data(), sizeof(int32_t) * plan.tu.start.size());
    put(ch.o_tv_start, plan.tv.start.data(), sizeof(int32_t) * plan.tv.start.size());
    put(ch.o_tu_of, plan.tu.of.data(), sizeof(int32_t) * plan.tu.of.size());
    put(ch.o_tv_of, plan.tv.of.data(), sizeof(int32_t) * plan.tv.of.size());
    // the staging vectors are pageable: wait before they go out of scope
    cuda_check(cudaStreamSynchronize(stream_), "upload");

    win_rows_ = std::max(win_rows_, ch.win_rows);
    win_cols_ = std::max(win_cols_, ch.win_cols);
    info_.visibilities += ch.M;
    info_.pixels += int64_t(ch.Nx) * ch.Ny;
  }
  ntasks_ = int(tasks.size());
  info_.win_rows = win_rows_;
  info_.win_cols = win_cols_;
  info_.channels = nch_;
  info_.tasks = ntasks_;

  // Channels of one grid size share a batched FFT plan over contiguous grids.
  for (int c = 0; c < nch_; ++c) {
    int g = 0;
    while (g < int(groups_.size()) &&
           !(groups_[g].Nu == chans_[c].Nu && groups_[g].Nv == chans_[c].Nv))
      ++g;
    if (g == int(groups_.size())) {
      groups_.emplace_back();
      groups_[g].Nu = chans_[c].Nu;
      groups_[g].Nv = chans_[c].Nv;
    }
    chans_[c].group = g;
    chans_[c].in_group = int(groups_[g].chans.size());
    groups_[g].chans.push_back(c);
  }
  info_.size_groups = int(groups_.size());
  for (SizeGroup &g : groups_) {
    g.fused = std::is_same<real, float>::value && fft_rows_supported(g.Nu);
    g.ld = g.fused ? g.Nu * int(g.chans.size()) : g.Nu;
    for (int c : g.chans) g.max_ny = std::max(g.max_ny, chans_[c].Ny);
    const size_t gb = sizeof(C) * size_t(g.Nu) * g.Nv * g.chans.size();
    g.o_pad = shared_.reserve(gb);
    g.o_work = shared_.reserve(gb);
    if (g.fused) {
      g.own_cols = cfg.fft_columns != 1 && fft_cols_supported(g.Nv, g.ld);
      g.o_members = shared_.reserve(sizeof(int) * g.chans.size());
      g.o_tw = shared_.reserve(2 * sizeof(float) * size_t(g.Nu));
      g.o_twv = shared_.reserve(2 * sizeof(float) * size_t(g.Nv));
    }
  }
  for (int c = 0; c < nch_; ++c) {
    const Chan &ch = chans_[c];
    const int64_t npix = (int64_t(ch.Nx) * ch.Ny + kGroupPixels - 1) / kGroupPixels;
    for (int64_t k = 0; k < npix; ++k) map_pix_.push_back(int2{c, int(k)});
    if (!groups_[ch.group].fused)
      for (int64_t k = 0; k < npix; ++k) map_pad_.push_back(int2{c, int(k)});
    const int64_t nsl = (ch.S + kGroupSlots - 1) / kGroupSlots;
    for (int64_t k = 0; k < nsl; ++k) map_slot_.push_back(int2{c, int(k)});
    for (int k = 0; k < ch.ntu * ch.ntv; ++k) map_tile_.push_back(int2{c, k});
    if (!ch.unit)
      for (int64_t k = 0; k < (ch.M + kGroupSlots - 1) / kGroupSlots; ++k)
        map_wvis_.push_back(int2{c, int(k)});
  }
  o_map_pix_ = shared_.reserve(sizeof(int2) * map_pix_.size());
  o_map_pad_ = shared_.reserve(sizeof(int2) * map_pad_.size());
  o_map_slot_ = shared_.reserve(sizeof(int2) * map_slot_.size());
  o_map_tile_ = shared_.reserve(sizeof(int2) * map_tile_.size());
  o_map_wvis_ = shared_.reserve(sizeof(int2) * map_wvis_.size());
  o_order_ = shared_.reserve(sizeof(int32_t) * order.size());
  o_tasks_ = shared_.reserve(sizeof(Task) * tasks.size());
  o_task_base_ = shared_.reserve(sizeof(int32_t) * nch_);
  o_fwd_ = shared_.reserve(sizeof(ApplyArgs<real>) * nch_);
  o_adj_ = shared_.reserve(sizeof(ApplyArgs<real>) * nch_);
  o_folds_ = shared_.reserve(sizeof(FoldArgs) * nch_);
  o_io_ = shared_.reserve(sizeof(ChannelIO<real>) * nch_);
  o_partial_ = shared_.reserve(sizeof(double) * kNormBlocks * nch_);
  o_sq_ = shared_.reserve(sizeof(double) * nch_);
  o_inv_ = shared_.reserve(sizeof(double) * nch_);
  shared_.allocate(&info_.device_bytes);
  for (const SizeGroup &g : groups_)
    cuda_check(cudaMemsetAsync(shared_.at<char>(g.o_pad), 0,
                               sizeof(C) * size_t(g.Nu) * g.Nv * g.chans.size(), stream_),
               "cudaMemset");
  if (!tasks.empty()) {
    cuda_check(cudaMemcpyAsync(shared_.at<char>(o_tasks_), tasks.data(), sizeof(Task) * tasks.size(),
                               cudaMemcpyHostToDevice, stream_),
               "upload");
    cuda_check(cudaMemcpyAsync(shared_.at<char>(o_order_), order.data(),
                               sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice, stream_),
               "upload");
  }
  cuda_check(cudaMemcpyAsync(shared_.at<char>(o_task_base_), task_base.data(),
                             sizeof(int32_t) * nch_, cudaMemcpyHostToDevice, stream_),
             "upload");
  for (auto m : {std::make_pair(&map_pix_, o_map_pix_), std::make_pair(&map_pad_, o_map_pad_),
                 std::make_pair(&map_slot_, o_map_slot_),
                 std::make_pair(&map_tile_, o_map_tile_), std::make_pair(&map_wvis_, o_map_wvis_)})
    if (!m.first->empty())
      cuda_check(cudaMemcpyAsync(shared_.at<char>(m.second), m.first->data(),
                                 sizeof(int2) * m.first->size(), cudaMemcpyHostToDevice, stream_),
                 "upload");
  for (SizeGroup &g : groups_) {
    if (g.fused) {
      // columns of the interleaved group: ld columns of Nv cells, stride ld
      if (!g.own_cols) {
        g.fft = make_column_plan<real>(g.ld, g.Nv, stream_, &info_.device_bytes);
        g.fft_ok = true;
      }
      const std::vector<float> twv = fft_twiddles(g.Nv);
      cuda_check(cudaMemcpyAsync(shared_.at<char>(g.o_twv), twv.data(), sizeof(float) * twv.size(),
                                 cudaMemcpyHostToDevice, stream_),
                 "upload");
      cuda_check(cudaMemcpyAsync(shared_.at<char>(g.o_members), g.chans.data(),
                                 sizeof(int) * g.chans.size(), cudaMemcpyHostToDevice, stream_),
                 "upload");
      const std::vector<float> tw = fft_twiddles(g.Nu);
      cuda_check(cudaMemcpyAsync(shared_.at<char>(g.o_tw), tw.data(), sizeof(float) * tw.size(),
                                 cudaMemcpyHostToDevice, stream_),
                 "upload");
      // the pageable sources above must outlive their staging
      cuda_check(cudaStreamSynchronize(stream_), "upload");
      continue;
    }
    int n[2] = {g.Nv, g.Nu};
    const int dist = g.Nu * g.Nv;
    cufft_check(cufftPlanMany(&g.fft, 2, n, nullptr, 1, dist, nullptr, 1, dist,
                              Traits<real>::kType, int(g.chans.size())),
                "cufftPlanMany");
    g.fft_ok = true;
    cufft_check(cufftSetStream(g.fft, stream_), "cufftSetStream");
    size_t ws = 0;
    if (cufftGetSize(g.fft, &ws) == CUFFT_SUCCESS) info_.device_bytes += int64_t(ws);
  }

  // Argument tables (I/O pointers are filled in by bind()).
  fwd_.resize(nch_);
  adj_.resize(nch_);
  folds_.resize(nch_);
  io_.resize(nch_);
  for (int c = 0; c < nch_; ++c) {
    Chan &ch = chans_[c];
    const Arena &m = ch.mem;
    ApplyArgs<real> a;
    a.batches = m.at<int2>(ch.o_batches);
    a.lane_code = m.at<int32_t>(ch.o_lane);
    a.frac = m.at<char>(ch.o_frac);
    a.Nu = ch.Nu;
    a.Nv = ch.Nv;
    a.ld = groups_[ch.group].ld;
    a.win_stride = ch.win_stride;
    a.group_cells = cfg_group_;
    a.slot_stride = ch.slot_stride;
    // forward: degrid straight into the caller-ordered visibilities
    fwd_[c] = a;
    fwd_[c].grid = work_of(c);
    fwd_[c].slot_user = m.at<int32_t>(ch.o_slot_user);
    // adjoint: visibilities gathered into slot order first
    adj_[c] = a;
    adj_[c].tilebuf = m.at<char>(ch.o_tilebuf);
    adj_[c].slot_in = m.at<char>(ch.o_slots);
    FoldArgs &f = folds_[c];
    f.tilebuf = m.at<char>(ch.o_tilebuf);
    f.slot_stride = ch.slot_stride;
    f.tile_tasks = m.at<int32_t>(ch.o_tile_tasks);
    f.tu_start = m.at<int32_t>(ch.o_tu_start);
    f.tv_start = m.at<int32_t>(ch.o_tv_start);
    f.tu_of = m.at<int32_t>(ch.o_tu_of);
    f.tv_of = m.at<int32_t>(ch.o_tv_of);
    f.ntu = ch.ntu;
    f.ntv = ch.ntv;
    // windows reach a block's extent - 1 cells into the next tiles
    f.Ju = J_ + group_u(cfg_group_) - 1;
    f.Jv = J_ + group_v(cfg_group_) - 1;
    f.Nu = ch.Nu;
    f.Nv = ch.Nv;
    f.ld = groups_[ch.group].ld;
    f.grid = work_of(c);
    ChannelIO<real> &io = io_[c];
    io.su = m.at<real>(ch.o_su);
    io.sv = m.at<real>(ch.o_sv);
    io.pad = pad_of(c);
    io.work = work_of(c);
    io.slots = m.at<char>(ch.o_slots);
    io.slot_user = m.at<int32_t>(ch.o_slot_user);
    io.user_slot = m.at<int32_t>(ch.o_user_slot);
    io.w_slot = ch.unit ? nullptr : m.at<char>(ch.o_weight);
    io.w_vis = ch.unit ? nullptr : m.at<char>(ch.o_wvis);
    io.Nx = ch.Nx;
    io.Ny = ch.Ny;
    io.Nu = ch.Nu;
    io.Nv = ch.Nv;
    io.ld = groups_[ch.group].ld;
    io.x0 = ch.x0;
    io.y0 = ch.y0;
    io.M = ch.M;
    io.S = ch.S;
  }
  bound_x_in_.assign(nch_, nullptr);
  bound_vis_.assign(nch_, nullptr);
  bound_x_out_.assign(nch_, nullptr);
  upload_tables(stream_);
  upload_corrections();
  cuda_check(cudaStreamSynchronize(stream_), "batch setup");
}

template <typename real>
BatchT<real>::~BatchT() {
  if (stream_) cudaStreamSynchronize(stream_);
  drop_graphs();
  for (SizeGroup &g : groups_)
    if (g.fft_ok) cufftDestroy(g.fft);
  if (ev_in_) cudaEventDestroy(ev_in_);
  if (ev_out_) cudaEventDestroy(ev_out_);
  if (stream_) cudaStreamDestroy(stream_);
}

// Phi_c = G F Z S / norm_c with a unitary F: 1 / (sqrt(Nu Nv) norm_c) is folded
// into the correction factors of each channel.
template <typename real>
void BatchT<real>::upload_corrections() {
  for (int k = 0; k < nch_; ++k) {
    Chan &ch = chans_[k];
    const double c = 1.0 / (std::sqrt(double(ch.Nu) * double(ch.Nv)) * ch.norm);
    std::vector<real> su(ch.Nx), sv(ch.Ny);
    for (int i = 0; i < ch.Nx; ++i) su[i] = real(ch.su[i] * c);
    for (int j = 0; j < ch.Ny; ++j) sv[j] = real(ch.sv[j]);
    cuda_check(cudaMemcpyAsync(ch.mem.template at<char>(ch.o_su), su.data(), sizeof(real) * ch.Nx,
                               cudaMemcpyHostToDevice, stream_),
               "correction upload");
    cuda_check(cudaMemcpyAsync(ch.mem.template at<char>(ch.o_sv), sv.data(), sizeof(real) * ch.Ny,
                               cudaMemcpyHostToDevice, stream_),
               "correction upload");
    cuda_check(cudaStreamSynchronize(stream_), "correction upload");
  }
}

// The tables are copied from pageable host memory: cudaMemcpyAsync returns
// once the source has been staged, and the copy is ordered on `s` before any
// later replay.
template <typename real>
void BatchT<real>::upload_tables(cudaStream_t s) {
  for (int c = 0; c < nch_; ++c) {
    fwd_[c].slot_out = bound_vis_[c];
    io_[c].x_in = bound_x_in_[c];
    io_[c].x_out = bound_x_out_[c];
    io_[c].vis_in = bound_vis_[c];
    io_[c].vis_out = bound_vis_[c];
  }
  cuda_check(cudaMemcpyAsync(shared_.at<char>(o_fwd_), fwd_.data(), sizeof(ApplyArgs<real>) * nch_,
                             cudaMemcpyHostToDevice, s),
             "table upload");
  cuda_check(cudaMemcpyAsync(shared_.at<char>(o_adj_), adj_.data(), sizeof(ApplyArgs<real>) * nch_,
                             cudaMemcpyHostToDevice, s),
             "table upload");
  cuda_check(cudaMemcpyAsync(shared_.at<char>(o_folds_), folds_.data(), sizeof(FoldArgs) * nch_,
                             cudaMemcpyHostToDevice, s),
             "table upload");
  cuda_check(cudaMemcpyAsync(shared_.at<char>(o_io_), io_.data(), sizeof(ChannelIO<real>) * nch_,
                             cudaMemcpyHostToDevice, s),
             "table upload");
}

template <typename real>
void BatchT<real>::join(cudaStream_t user) {
  cuda_check(cudaEventRecord(ev_in_, user), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(stream_, ev_in_, 0), "cudaStreamWaitEvent");
}
template <typename real>
void BatchT<real>::release(cudaStream_t user) {
  cuda_check(cudaEventRecord(ev_out_, stream_), "cudaEventRecord");
  cuda_check(cudaStreamWaitEvent(user, ev_out_, 0), "cudaStreamWaitEvent");
}

// The launches of one step, in stream order on stream_.
template <typename real>
void BatchT<real>::record(int mode) {
  const ChannelIO<real> *io = shared_.at<ChannelIO<real>>(o_io_);
  ApplyArgs<real> head;
  head.group_cells = cfg_group_;
  head.tasks = shared_.at<Task>(o_tasks_);
  head.order = shared_.at<int32_t>(o_order_);
  head.group_task_base = shared_.at<int32_t>(o_task_base_);
  if (mode == kDegridOnly || mode == kGridOnly) {  // one gridding launch alone (timing)
    const bool dg = mode == kDegridOnly;
    head.group = shared_.at<ApplyArgs<real>>(dg ? o_fwd_ : o_adj_);
    cuda_check(dg ? launch_degrid_group<real>(head, poly_, J_, ntasks_, win_rows_, win_cols_,
                                              degrid_shape_, true, stream_)
                  : launch_grid_group<real>(head, poly_, J_, ntasks_, win_rows_, win_cols_,
                                            grid_shape_, false, stream_),
               dg ? "degrid" : "grid");
    return;
  }
  if (mode & kForward) {
    if (!map_pad_.empty())
      cuda_check(launch_pad_group<real>(io, shared_.at<int2>(o_map_pad_), int(map_pad_.size()),
                                        stream_),
                 "pad");
    for (SizeGroup &g : groups_) {
      if (g.fused) {
        // S, padding and the row FFT of every member's image rows into the
        // group's padded grid (its other rows stay zero), then the columns
        cuda_check(launch_fft_rows_group(false, io, shared_.at<int>(g.o_members),
                                         int(g.chans.size()), g.Nu, g.max_ny, g.ld,
                                         shared_.at<char>(g.o_tw), stream_),
                   "row pass");
        if (g.own_cols) {
          cuda_check(launch_fft_cols(false, col_args(g, false), stream_), "column pass");
          continue;
        }
      }
      cufft_check(Traits<real>::exec(g.fft, shared_.at<C>(g.o_pad), shared_.at<C>(g.o_work),
                                     CUFFT_FORWARD),
                  "cufftExec");
    }
    head.group = shared_.at<ApplyArgs<real>>(o_fwd_);
    cuda_check(launch_degrid_group<real>(head, poly_, J_, ntasks_, win_rows_, win_cols_,
                                         degrid_shape_, true, stream_),
               "degrid");
    cuda_check(launch_weigh_vis_group<real>(io, shared_.at<int2>(o_map_wvis_),
                                            int(map_wvis_.size()), stream_),
               "weights");
  }
  if (mode & kAdjoint) {
    cuda_check(launch_expand_group<real>(io, shared_.at<int2>(o_map_slot_), int(map_slot_.size()),
                                         stream_),
               "expand");
    head.group = shared_.at<ApplyArgs<real>>(o_adj_);
    cuda_check(launch_grid_group<real>(head, poly_, J_, ntasks_, win_rows_, win_cols_,
                                       grid_shape_, false, stream_),
               "grid");
    cuda_check(launch_fold_group<real>(shared_.at<FoldArgs>(o_folds_), shared_.at<int2>(o_map_tile_),
                                       int(map_tile_.size()), stream_),
               "fold");
    for (SizeGroup &g : groups_) {
      if (g.own_cols)
        cuda_check(launch_fft_cols(true, col_args(g, true), stream_), "column pass");
      else
        cufft_check(Traits<real>::exec(g.fft, shared_.at<C>(g.o_work), shared_.at<C>(g.o_work),
                                       CUFFT_INVERSE),
                    "cufftExec");
      if (g.fused)
        cuda_check(launch_fft_rows_group(true, io, shared_.at<int>(g.o_members),
                                         int(g.chans.size()), g.Nu, g.max_ny, g.ld,
                                         shared_.at<char>(g.o_tw), stream_),
                   "row pass");
    }
    if (!map_pad_.empty())
      cuda_check(launch_crop_group<real>(io, shared_.at<int2>(o_map_pad_), int(map_pad_.size()),
                                         stream_),
                 "crop");
  }
  if (mode == kPower)
    cuda_check(launch_sq_norm_group<real>(io, nch_, shared_.at<double>(o_partial_),
                                          shared_.at<double>(o_sq_), stream_),
               "norm");
}

// The column pass of a fused size group: forward pad -> work (reading each
// member's image rows only), inverse work -> work in place (writing them only).
template <typename real>
FftColArgs BatchT<real>::col_args(const SizeGroup &g, bool inverse) const {
  FftColArgs c;
  c.in = shared_.at<C>(inverse ? g.o_work : g.o_pad);
  c.out = shared_.at<C>(g.o_work);
  c.Nv = g.Nv;
  c.W = g.ld;
  c.ld = g.ld;
  c.tw_v = shared_.at<char>(g.o_twv);
  c.chans = shared_.at<char>(o_io_);
  c.members = shared_.at<int>(g.o_members);
  c.Nu = g.Nu;
  return c;
}

template <typename real>
cudaGraphExec_t BatchT<real>::graph_for(int mode) {
  auto it = graphs_.find(mode);
  if (it != graphs_.end()) return it->second.second;
  cudaGraph_t g = nullptr;
  cuda_check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "capture");
  try {
    record(mode);
  } catch (...) {
    cudaStreamEndCapture(stream_, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  cuda_check(cudaStreamEndCapture(stream_, &g), "capture");
  cudaGraphExec_t e = nullptr;
  const cudaError_t r = cudaGraphInstantiate(&e, g, 0);
  if (r != cudaSuccess) {
    cudaGraphDestroy(g);
    cuda_check(r, "cudaGraphInstantiate");
  }
  graphs_[mode] = {g, e};
  return e;
}

template <typename real>
void BatchT<real>::drop_graphs() {
  for (auto &kv : graphs_) {
    cudaGraphExecDestroy(kv.second.second);
    cudaGraphDestroy(kv.second.first);
  }
  graphs_.clear();
}

template <typename real>
void BatchT<real>::set_launch_shapes(int degrid_threads, int grid_threads) {
  for (int t : {degrid_threads, grid_threads})
    if (t % 32 != 0 || t < 32 || t > 256)
      throw Error(kInvalidArgument, "threads must be a multiple of 32 in [32, 256]");
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  cuda_check(cudaStreamSynchronize(stream_), "set_launch_shapes");
  drop_graphs();
  degrid_shape_.threads = degrid_threads;
  grid_shape_.threads = grid_threads;
}

template <typename real>
void BatchT<real>::bind_internal() {
  for (int c = 0; c < nch_; ++c) {
    Chan &ch = chans_[c];
    void *x = ch.mem.template at<char>(ch.o_pm_x);
    bound_x_in_[c] = x;
    bound_x_out_[c] = x;
    bound_vis_[c] = ch.mem.template at<char>(ch.o_pm_vis);
  }
  upload_tables(stream_);
}

template <typename real>
double BatchT<real>::time_apply(int directions, int reps) {
  if (!(directions == kForward || directions == kAdjoint || directions == kBoth ||
        directions == kDegridOnly || directions == kGridOnly) ||
      reps < 1)
    throw Error(kInvalidArgument, "time_apply: bad directions or repetitions");
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  const std::vector<const void *> saved_x_in = bound_x_in_;
  const std::vector<void *> saved_vis = bound_vis_, saved_x_out = bound_x_out_;
  cudaEvent_t a = nullptr, b = nullptr;
  double ms = 0;
  try {
    bind_internal();
    for (int c = 0; c < nch_; ++c) {
      const int64_t N = int64_t(chans_[c].Nx) * chans_[c].Ny;
      cuda_check(launch_fill<real>(bound_x_out_[c], N, 1.0 / std::sqrt(double(N)), stream_), "fill");
    }
    const cudaGraphExec_t e = graph_for(directions);
    cuda_check(cudaEventCreate(&a), "cudaEventCreate");
    cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    for (int k = 0; k < 2; ++k) cuda_check(cudaGraphLaunch(e, stream_), "cudaGraphLaunch");
    cuda_check(cudaEventRecord(a, stream_), "cudaEventRecord");
    for (int k = 0; k < reps; ++k) cuda_check(cudaGraphLaunch(e, stream_), "cudaGraphLaunch");
    cuda_check(cudaEventRecord(b, stream_), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(b), "cudaEventSynchronize");
    float f = 0;
    cuda_check(cudaEventElapsedTime(&f, a, b), "cudaEventElapsedTime");
    ms = double(f) / reps;
  } catch (...) {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    bound_x_in_ = saved_x_in;
    bound_vis_ = saved_vis;
    bound_x_out_ = saved_x_out;
    upload_tables(stream_);
    cudaStreamSynchronize(stream_);
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  bound_x_in_ = saved_x_in;
  bound_vis_ = saved_vis;
  bound_x_out_ = saved_x_out;
  upload_tables(stream_);
  cuda_check(cudaStreamSynchronize(stream_), "time_apply");
  return ms;
}

template <typename real>
void BatchT<real>::bind(const void *const *x_in, void *const *vis, void *const *x_out,
                        cudaStream_t user) {
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  for (int c = 0; c < nch_; ++c) {
    bound_x_in_[c] = x_in ? x_in[c] : nullptr;
    bound_vis_[c] = vis ? vis[c] : nullptr;
    bound_x_out_[c] = x_out ? x_out[c] : nullptr;
  }
  join(user);
  upload_tables(stream_);
  release(user);
}

template <typename real>
void BatchT<real>::apply(int directions, cudaStream_t user) {
  if (directions < 1 || directions > 3)
    throw Error(kInvalidArgument, "directions must be 1 (forward), 2 (adjoint) or 3 (both)");
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  for (int c = 0; c < nch_; ++c) {
    const bool vis_ok = bound_vis_[c] || chans_[c].M == 0;
    const bool fwd_ok = vis_ok && bound_x_in_[c];
    const bool adj_ok = vis_ok && bound_x_out_[c];
    if (((directions & kForward) && !fwd_ok) || ((directions & kAdjoint) && !adj_ok))
      throw Error(kInvalidArgument, "channel " + std::to_string(c) + " has no bound buffers");
  }
  const cudaGraphExec_t e = graph_for(directions);
  join(user);
  cuda_check(cudaGraphLaunch(e, stream_), "cudaGraphLaunch");
  release(user);
}

template <typename real>
void BatchT<real>::set_norms(const double *norms) {
  for (int c = 0; c < nch_; ++c)
    if (!(norms[c] > 0)) throw Error(kNormNotPositive, "Operator norm is not greater than zero.");
  DeviceGuard guard(device_);
  std::lock_guard<std::mutex> lock(mu_);
  cuda_check(cudaStreamSynchronize(stream_), "set_norms");
  for (int c = 0; c < nch_; ++c) chans_[c].norm = norms[c];
  upload_corrections();
}

template <typename real>
void BatchT<real>::get_norms(double *norms) const {
  for (int c = 0; c < nch_; ++c) norms[c] = chans_[c].norm;
}

// Power iteration of every channel at once, each channel following the
// single-operator rule (operators.h:390-391): start from the normalised
// all-ones image, estimate = FP64 2-norm of the iterate, stop when its
// relative change drops below tol^2, norm = sqrt(estimate).  A channel that
// has stopped keeps iterating with the others, but its result is the
// estimate at its own stopping step, so it does not depend on the batch.
template <typename real>
void BatchT<real>::power_method(int iters, double tol, double *norms_out) {
  DeviceGuard guard(device_);
  std::vector<double> result(nch_, 1.0);
  if (iters > 0) {
    std::lock_guard<std::mutex> lock(mu_);
    cuda_check(cudaStreamSynchronize(stream_), "power_method");
    const std::vector<double> saved_norm = [&] {
      std::vector<double> s(nch_);
      for (int c = 0; c < nch_; ++c) s[c] = chans_[c].norm;
      return s;
    }();
    const std::vector<const void *> saved_x_in = bound_x_in_;
    const std::vector<void *> saved_vis = bound_vis_, saved_x_out = bound_x_out_;
    auto restore = [&](bool norms_too) {
      bound_x_in_ = saved_x_in;
      bound_vis_ = saved_vis;
      bound_x_out_ = saved_x_out;
      upload_tables(stream_);
      if (norms_too) {
        for (int c = 0; c < nch_; ++c) chans_[c].norm = saved_norm[c];
        upload_corrections();
      }
      cuda_check(cudaStreamSynchronize(stream_), "power_method");
    };
    try {
      bind_internal();
      for (int c = 0; c < nch_; ++c) {
        Chan &ch = chans_[c];
        ch.norm = 1.0;
        const int64_t N = int64_t(ch.Nx) * ch.Ny;
        cuda_check(launch_fill<real>(bound_x_out_[c], N, 1.0 / std::sqrt(double(N)), stream_),
                   "fill");
      }
      upload_corrections();
      const cudaGraphExec_t e = graph_for(kPower);
      std::vector<double> sq(nch_), inv(nch_), old_value(nch_, 0.0);
      std::vector<char> done(nch_, 0);
      int remaining = nch_;
      for (int i = 0; i < iters && remaining > 0; ++i) {
        cuda_check(cudaGraphLaunch(e, stream_), "cudaGraphLaunch");
        cuda_check(cudaMemcpyAsync(sq.data(), shared_.at<char>(o_sq_), sizeof(double) * nch_,
                                   cudaMemcpyDeviceToHost, stream_),
                   "D2H");
        cuda_check(cudaStreamSynchronize(stream_), "power_method");
        for (int c = 0; c < nch_; ++c) {
          const double value = std::sqrt(sq[c]);
          if (!(value > 0)) {
            if (done[c]) {
              inv[c] = 1.0;
              continue;
            }
            throw Error(kNormNotPositive, "Operator norm is not greater than zero.");
          }
          inv[c] = 1.0 / value;
          if (done[c]) continue;
          if (tol * tol > std::abs(old_value[c] - value) / old_value[c]) {
            done[c] = 1;
            --remaining;
          }
          old_value[c] = value;
        }
        cuda_check(cudaMemcpyAsync(shared_.at<char>(o_inv_), inv.data(), sizeof(double) * nch_,
                                   cudaMemcpyHostToDevice, stream_),
                   "H2D");
        cuda_check(launch_scale_group<real>(shared_.at<ChannelIO<real>>(o_io_),
                                            shared_.at<int2>(o_map_pix_), int(map_pix_.size()),
                                            shared_.at<double>(o_inv_), stream_),
                   "scale");
      }
      for (int c = 0; c < nch_; ++c) result[c] = std::sqrt(old_value[c]);
    } catch (...) {
      restore(true);
      throw;
    }
    restore(false);
  }
  set_norms(result.data());
  if (norms_out)
    for (int c = 0; c < nch_; ++c) norms_out[c] = result[c];
}

}  // namespace

std::unique_ptr<Batch> Batch::create(const BatchConfig &cfg) {
  if (cfg.channels.empty()) throw Error(kInvalidArgument, "a batch needs at least one channel");
  if (!(cfg.oversample_ratio >= 1.0))
    throw Error(kInvalidArgument, "oversample_ratio must be >= 1");
  const std::string why = check_kernel_request(cfg.kernel, cfg.J, cfg.J);
  if (!why.empty()) throw Error(kInvalidArgument, why);
  if (cfg.J < 1 || cfg.J > kMaxJ)
    throw Error(kUnsupported, "kernel support must be between 1 and 8 taps");
  for (int t : {cfg.threads, cfg.degrid_threads, cfg.grid_threads})
    if (t != 0 && (t % 32 != 0 || t < 32 || t > 256))
      throw Error(kInvalidArgument, "threads must be a multiple of 32 in [32, 256]");
  if (cfg.threads == 0) throw Error(kInvalidArgument, "threads must be given");
  if (cfg.tile < 8 || cfg.tile > 128) throw Error(kInvalidArgument, "tile must be in [8, 128]");
  if (cfg.max_per_item < 1 || cfg.max_per_item > 64)
    throw Error(kInvalidArgument, "max_per_item must be in [1, 64]");
  if (cfg.cell_group < 1 || cfg.cell_group > 3)
    throw Error(kInvalidArgument, "cell_group must be 1, 2 or 3");
  if (cfg.cell_group >= 2 && (cfg.fp64 || cfg.J > kMaxGroupJ))
    throw Error(kUnsupported, "2 x 2 work items need complex<float> and J <= 6");
  for (size_t c = 0; c < cfg.channels.size(); ++c) {
    const ChannelSpec &s = cfg.channels[c];
    if (s.imsizex <= 0 || s.imsizey <= 0)
      throw Error(kInvalidArgument, "channel " + std::to_string(c) + ": empty image");
    if (s.M < 0)
      throw Error(kInvalidArgument, "channel " + std::to_string(c) + ": negative visibilities");
    if (s.M > 0 && (!s.u || !s.v))
      throw Error(kInvalidArgument, "channel " + std::to_string(c) + ": u and v must be given");
  }
  if (cfg.fp64) return std::unique_ptr<Batch>(new BatchT<double>(cfg));
  return std::unique_ptr<Batch>(new BatchT<float>(cfg));
}

namespace {
std::mutex g_tune_mu;
std::map<std::string, BatchTuning> g_tune_cache;
}  // namespace

BatchTuning autotune_batch(const BatchConfig &cfg) {
  const int n = int(cfg.channels.size());
  if (n == 0) throw Error(kInvalidArgument, "a batch needs at least one channel");
  // Sample: up to eight channels evenly spaced in visibility count.
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return cfg.channels[a].M < cfg.channels[b].M; });
  const int K = std::min(n, 8);
  BatchConfig sub = cfg;
  sub.channels.clear();
  std::ostringstream key;
  key << cfg.fp64 << ':' << cfg.kernel << ':' << cfg.J << ':' << cfg.oversample_ratio << ':'
      << cfg.max_per_item << ':' << cfg.device;
  for (int k = 0; k < K; ++k) {
    const int c = order[K == 1 ? n / 2 : int(int64_t(k) * (n - 1) / (K - 1))];
    const ChannelSpec &spec = cfg.channels[c];
    sub.channels.push_back(spec);
    key << '|' << spec.imsizey << 'x' << spec.imsizex << ':'
        << (spec.M > 0 ? int(std::lround(4.0 * std::log2(double(spec.M)))) : -1);
  }
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(key.str());
    if (it != g_tune_cache.end()) return it->second;
  }
  int optin = 0;
  cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cfg.device),
             "cudaDeviceGetAttribute");
  const int prec = cfg.fp64 ? 8 : 4;
  // sub-segments of the tap fit (their coefficients take shared memory)
  const int nsub = fit_axis(GriddingKernel(cfg.kernel, cfg.J, cfg.oversample_ratio), cfg.J,
                            cfg.fp64 ? kCoefF64 : kCoefF32).nsub;
  BatchTuning best;
  double best_ms = -1;
  const int max_group = (!cfg.fp64 && cfg.J <= kMaxGroupJ) ? 2 : 1;
  for (int group = 1; group <= max_group; ++group)
  for (int tile : {24, 32, 48}) {
    sub.tile = tile;
    sub.cell_group = group;
    sub.threads = 128;
    sub.degrid_threads = sub.grid_threads = 0;
    std::unique_ptr<Batch> b = Batch::create(sub);
    const BatchInfo bi = b->info();
    double fwd_best = -1, adj_best = -1;
    int fwd_t = 0, adj_t = 0;
    for (int threads : {64, 128, 256}) {
      LaunchShape shape;
      shape.threads = threads;
      const bool degrid_fits =
          degrid_smem_bytes(prec, cfg.J, bi.win_rows, bi.win_cols, shape, true, group, nsub) <=
          size_t(optin);
      const bool grid_fits =
          grid_smem_bytes(prec, cfg.J, bi.win_rows, bi.win_cols, shape, false, group, nsub) <=
          size_t(optin);
      if (!degrid_fits || !grid_fits) continue;
      b->set_launch_shapes(threads, threads);
      const double f = b->time_apply(1, 5), a = b->time_apply(2, 5);
      if (fwd_best < 0 || f < fwd_best) {
        fwd_best = f;
        fwd_t = threads;
      }
      if (adj_best < 0 || a < adj_best) {
        adj_best = a;
        adj_t = threads;
      }
    }
    if (fwd_t == 0 || adj_t == 0) continue;
    if (best_ms < 0 || fwd_best + adj_best < best_ms) {
      best_ms = fwd_best + adj_best;
      best.tile = tile;
      best.cell_group = group;
      best.max_per_item = cfg.max_per_item;
      best.degrid_threads = fwd_t;
      best.grid_threads = adj_t;
    }
  }
  if (best_ms < 0) throw Error(kUnsupported, "no tile / CTA shape fits in shared memory");
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune_cache[key.str()] = best;
  return best;
}

}  // namespace pg
