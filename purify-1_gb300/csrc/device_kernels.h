// Host-callable launchers of the sm_103a kernels.  Plain C++ declarations so
// that host translation units compiled by g++ can call them.
#pragma once
#include <cuda_runtime_api.h>

#include <cstddef>
#include <cstdint>

#include "pg_types.h"

namespace pg {

// Pointers and sizes of one coverage plus the I/O buffers of one apply.
// Complex arrays hold interleaved (re, im) pairs of `real`.  Visibility
// vectors here are in slot order (see plan.h).
template <typename real>
struct ApplyArgs {
  const void *grid = nullptr;       // degrid input: Nv x Nu complex
  void *tilebuf = nullptr;          // grid output: one window per task
  const Task *tasks = nullptr;
  const int2 *batches = nullptr;    // {first slot, kmax}
  const int32_t *lane_code = nullptr;  // item_pack per batch lane
  const void *frac = nullptr;       // S x (t_u, t_v); sign of t_u = the phase flip (-1)^(k_u + k_v)
  void *slot_out = nullptr;         // degrid output, S complex
  const void *slot_in = nullptr;    // grid input, S complex
  // When set, visibilities are read / written in caller order directly:
  // slot s holds visibility slot_user[s] (-1 = null slot), slot_out and
  // slot_in then point at caller-ordered M-vectors.
  const int32_t *slot_user = nullptr;
  int Nu = 0, Nv = 0;
  int ld = 0;                       // row stride of the grid in cells (0: Nu)
  int win_stride = 0;               // row stride of the shared-memory windows (plan's win_stride)
  int group_cells = 1;              // cells per work item along each axis (plan's group)
  // caller order (slot_user set): the grid kernel gathers and the degrid
  // kernel stores the caller-ordered vector at L2 evict-last priority, so it
  // stays in L2 between the two
  int keep_in = 0;
  int64_t slot_stride = 0;          // complex elements per tilebuf slot
  int win_bytes = 0;    // set by the launchers: shared bytes before the batch headers
  // set by the launchers: degrid, the per-warp staging stride; normal, the
  // shared bytes of the grid window before the warp windows
  int stage_bytes = 0;
  // Grouped launch over several operators: a device array of per-operator
  // ApplyArgs (indexed by Task::channel) and the first task of each operator
  // in the grouped task list (its tilebuf holds windows from that index on).
  const void *group = nullptr;
  // Launch order: CTA b runs task order[b] (longest tasks first, so the last
  // wave is short), or task b when null.
  const int32_t *order = nullptr;
  const int32_t *group_task_base = nullptr;
};

// Blocks of the first stage of the deterministic norm reductions.
constexpr int kNormBlocks = 512;

struct LaunchShape {
  int threads = 128;  // 32 x warps per CTA
};

// Largest dynamic shared memory a launch of the given shape needs, in bytes:
// user = visibilities in caller order (it sizes the degrid kernel's staging
// buffers; the grid kernel has none).
// nsub > 1 adds the tap coefficients the kernels copy into shared memory.
size_t degrid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                         const LaunchShape &shape, bool user = true, int group = 1,
                         int nsub = 1);
size_t grid_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                       const LaunchShape &shape, bool user = false, int group = 1,
                       int nsub = 1);

// G: tiles of the grid -> visibilities.
template <typename real>
cudaError_t launch_degrid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                          int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                          cudaStream_t s);
// G^H G of the normal operator in one pass (unit weights): the grid at a.grid
// -> one accumulated window per task at a.tilebuf, as launch_grid leaves
// them for the slot-ordered output of launch_degrid.
template <typename real>
cudaError_t launch_normal(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                          int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                          cudaStream_t s);
// Shared memory of launch_normal, or 0 where it does not apply (FP32,
// single-cell items, J <= 6).
size_t normal_smem_bytes(int precision_bytes, int J, int win_rows, int win_cols,
                         const LaunchShape &shape, int group, int nsub = 1);
// G^H, first half: visibilities -> one accumulated window per task.
template <typename real>
cudaError_t launch_grid(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                        int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                        cudaStream_t s);

// The same half of G^H on the column-walk plan (plan.h WalkPlan): slot-ordered
// visibilities in, one window per task out, in the layout the fold reads.
template <typename real>
struct WalkArgs {
  const Task *tasks = nullptr;
  const int32_t *order = nullptr;     // launch order of the tasks
  const int32_t *counts = nullptr;    // tasks x 32 columns x 32 rows
  const int32_t *colstart = nullptr;  // tasks x 33
  const void *frac = nullptr;         // S x (t_u, t_v), the phase flip in the sign of t_u
  const void *slot_in = nullptr;      // S complex, slot order
  void *tilebuf = nullptr;            // one window per task, slot_stride cells apart
  int64_t slot_stride = 0;
  int win_stride = 0;                 // odd
  int win_rows = 0;                   // rows of the largest window
  int max_steps = 0;                  // capacity of a warp's step list (plan's max_warp_steps)
};
template <typename real>
cudaError_t launch_walk_grid(const WalkArgs<real> &a, const PolyTable<real> &poly, int J,
                             int ntasks, int threads, cudaStream_t s);
// Shared memory of a column-walk CTA: kWalkWarps windows of win_rows x
// win_stride cells, and per warp a list of max_steps steps and its column
// offsets into it.
// With nsub > 1 the tap coefficients follow, from the next 16-byte boundary
// (walk_coefficient_offset).
PG_HD inline size_t walk_coefficient_offset(int precision_bytes, int win_rows, int win_stride,
                                            int max_steps) {
  const size_t b = size_t(kWalkWarps) * (size_t(win_rows) * win_stride * 2 * precision_bytes +
                                         size_t(max_steps) * 8 + 9 * 4);
  return (b + 15) / 16 * 16;
}
inline size_t walk_smem_bytes(int precision_bytes, int win_rows, int win_stride, int max_steps,
                              int J = 1, int nsub = 1) {
  const size_t nc = precision_bytes == 8 ? 17 : 9;  // PolyCount<double>, PolyCount<float>
  return walk_coefficient_offset(precision_bytes, win_rows, win_stride, max_steps) +
         (nsub > 1 ? size_t(J) * nsub * nc * precision_bytes : 0);
}

// Grouped forms: `a.tasks` lists the tasks of several operators (Task::channel
// names the operator), `a.group` points at a device array of their ApplyArgs
// and `a.group_task_base` at the first grouped task of each; win_rows /
// win_cols are the largest over the group; user says whether any operator
// of the group reads or writes caller order.
template <typename real>
cudaError_t launch_degrid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                                int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                                bool user, cudaStream_t s);
template <typename real>
cudaError_t launch_grid_group(const ApplyArgs<real> &a, const PolyTable<real> &poly, int J,
                              int ntasks, int win_rows, int win_cols, const LaunchShape &shape,
                              bool user, cudaStream_t s);

// G^H, second half: sums the task windows that cover each grid cell, in a
// fixed order, into the grid.
struct FoldArgs {
  const void *tilebuf;
  int64_t slot_stride;
  const int32_t *tile_tasks;         // ntiles + 1
  const int32_t *tu_start, *tv_start;  // ntu + 1, ntv + 1
  const int32_t *tu_of, *tv_of;      // Nu, Nv
  int ntu, ntv, Ju, Jv, Nu, Nv;
  void *grid;
  int ld = 0;  // row stride of the grid in cells (0: Nu)
};
template <typename real>
cudaError_t launch_fold(const FoldArgs &f, cudaStream_t s);

// Per-operator arguments of the grouped element-wise kernels (batch of
// channels, one CTA row per channel).
template <typename real>
struct ChannelIO {
  const void *x_in = nullptr;   // image in (forward)
  void *x_out = nullptr;        // image out (adjoint)
  const real *su = nullptr, *sv = nullptr;
  void *pad = nullptr;          // zero-padded grid (forward FFT input)
  void *work = nullptr;         // FFT output / adjoint grid
  const void *vis_in = nullptr; // caller-ordered visibilities in (adjoint)
  void *vis_out = nullptr;      // caller-ordered visibilities out (forward)
  void *slots = nullptr;        // slot-ordered buffer
  const int32_t *slot_user = nullptr, *user_slot = nullptr;
  // weights (null for unit weights): w_slot in slot order (S values), used
  // conjugated by the gather before G^H; w_vis in caller order (M values),
  // multiplied into the forward's output
  const void *w_slot = nullptr, *w_vis = nullptr;
  int Nx = 0, Ny = 0, Nu = 0, Nv = 0, x0 = 0, y0 = 0;
  int ld = 0;  // row stride of pad and work in cells (0: Nu)
  int64_t M = 0, S = 0;
};

// Grouped element-wise launches run over a block map (one int2 {channel,
// block of that channel} per CTA): pad / crop / scale take kGroupPixels
// pixels per block, expand kGroupSlots slots, fold one tile.
constexpr int kGroupPixels = 256;
constexpr int kGroupSlots = 4 * 256;
template <typename real>
cudaError_t launch_pad_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                             cudaStream_t s);
template <typename real>
cudaError_t launch_crop_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                              cudaStream_t s);
template <typename real>
cudaError_t launch_expand_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                                cudaStream_t s);
// vis_out <- vis_out * w_vis over a block map of kGroupSlots visibilities
// per block (channels with weights only).
template <typename real>
cudaError_t launch_weigh_vis_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                                   cudaStream_t s);
// Per-channel deterministic FP64 sum of |x_out|^2 into out[c] (partial holds
// nch * kNormBlocks doubles), and x_out <- x_out * inv[c].
template <typename real>
cudaError_t launch_sq_norm_group(const ChannelIO<real> *chans, int nch, double *partial,
                                 double *out, cudaStream_t s);
template <typename real>
cudaError_t launch_scale_group(const ChannelIO<real> *chans, const int2 *map, int nblocks,
                               const double *inv, cudaStream_t s);
template <typename real>
cudaError_t launch_fold_group(const FoldArgs *folds, const int2 *map, int nblocks, cudaStream_t s);

// Z S: scaled gridding correction and zero padding.  su[i] sv[j] x[j Nx + i]
// lands at grid[(y0 + j) Nu + x0 + i]; other grid cells are left untouched.
template <typename real>
cudaError_t launch_pad(const void *x, const real *su, const real *sv, void *grid, int Nx, int Ny,
                       int Nu, int x0, int y0, cudaStream_t s);
// S^H Z^H: crop and scaled correction.
template <typename real>
cudaError_t launch_crop(const void *grid, const real *su, const real *sv, void *x, int Nx, int Ny,
                        int Nu, int x0, int y0, cudaStream_t s);

// Caller order <-> slot order.  compact: out[m] = slots[user_slot[m]], m < M.
// expand: slots[s] = in[slot_user[s]] (0 where slot_user[s] < 0), s < S.
// With keep_in, expand reads `in` at L2 evict-last priority, so the
// caller-ordered vector stays in L2 afterwards (for a vector that fits in it:
// the next degrid's scattered stores into it then hit L2).
template <typename real>
cudaError_t launch_compact(const void *slots, const int32_t *user_slot, void *out, int64_t M,
                           cudaStream_t s);
// With w (S complex values in slot order), slots[s] = conj(w[s]) in[...]:
// the conjugated weights of G^H applied in the same pass.
template <typename real>
cudaError_t launch_expand(const void *in, const int32_t *slot_user, void *slots, int64_t S,
                          cudaStream_t s, bool keep_in = false, const void *w = nullptr);

// complex<double> <-> complex<real> conversion of n values.
template <typename real>
cudaError_t launch_from_c128(const void *src, void *dst, int64_t n, cudaStream_t s);
template <typename real>
cudaError_t launch_to_c128(const void *src, void *dst, int64_t n, cudaStream_t s);

// Deterministic FP64 sum of |x|^2 over n complex values into *out (device).
// `partial` must hold kNormBlocks doubles.
template <typename real>
cudaError_t launch_sq_norm(const void *x, int64_t n, double *partial, double *out,
                           cudaStream_t s);
// x <- x * scale.
template <typename real>
cudaError_t launch_scale(void *x, int64_t n, double scale, cudaStream_t s);
// x <- x * real(1 / sqrt(*sq)) with *sq on the device (0 when not positive).
template <typename real>
cudaError_t launch_scale_rsqrt(void *x, int64_t n, const double *sq, cudaStream_t s);
// a <- a * b * scale, complex element-wise.
template <typename real>
cudaError_t launch_cmul_scale(void *a, const void *b, int64_t n, double scale, cudaStream_t s);
// a <- a * b, or a * conj(b) with conj_b, complex element-wise.
template <typename real>
cudaError_t launch_cmul(void *a, const void *b, int64_t n, bool conj_b, cudaStream_t s);
// x <- the unit vector e_index.
template <typename real>
cudaError_t launch_delta(void *x, int64_t n, int64_t index, cudaStream_t s);
// x <- value (complex, real part only).
template <typename real>
cudaError_t launch_fill(void *x, int64_t n, double value, cudaStream_t s);

}  // namespace pg
