/*
 * purify_gb300.h — C ABI of the GB300 measurement operator.
 *
 * The operator is PURIFY's Phi = G F Z S / ||Phi'||: gridding correction S,
 * zero padding Z, an oversampled unitary FFT F and Kaiser-Bessel (or other
 * kernel) degridding G, plus its adjoint.  It replaces the serial and GPU
 * slots of the reference's operator factory:
 *
 *   measurementoperator::init_degrid_operator_2d   cpp/purify/operators.h:372-414
 *   gpu::measurementoperator::init_degrid_operator_2d  cpp/purify/operators_gpu.h:292-332
 *   factory::measurement_operator_factory (gpu_serial)  cpp/purify/measurement_operator_factory.h:38-96
 *
 * Conventions (those of the reference):
 *   image vectors  imsizey x imsizex, index j * imsizex + i (row j is v/y)
 *   grid           ftsizev x ftsizeu with ftsize = floor(oversample * imsize)
 *   u, v           visibility coordinates in grid pixels (the "raw" overload);
 *                  purify_gb300_lambda_to_pixels converts from wavelengths
 *   complex data   interleaved (re, im); c128 = double pairs, c64 = float pairs
 *   precision      PURIFY_GB300_FP32 computes with complex<float> buffers (c64
 *                  device I/O), PURIFY_GB300_FP64 with complex<double> (c128)
 *
 * Every function returns a purify_gb300_status; on failure
 * purify_gb300_last_error() holds a message for the calling thread.  Nothing
 * throws across this boundary.  Applies of one operator are ordered on an
 * internal CUDA stream (joined to the caller's stream by events), so one
 * operator may be shared by threads.
 */
#ifndef PURIFY_GB300_H
#define PURIFY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  PURIFY_GB300_OK = 0,
  PURIFY_GB300_INVALID_ARGUMENT = 1, /* reference: std::runtime_error on sizes (operators.cc:18-20) */
  PURIFY_GB300_UNSUPPORTED = 2,
  PURIFY_GB300_CUDA_ERROR = 3,
  PURIFY_GB300_OUT_OF_MEMORY = 4,
  PURIFY_GB300_NORM_NOT_POSITIVE = 5, /* reference: init_normalise, operators.h:185-189 */
  PURIFY_GB300_REJECTED = 6,          /* serving: request refused by admission control */
  PURIFY_GB300_TIMEOUT = 7,
  PURIFY_GB300_INTERNAL = 8
} purify_gb300_status;

/* Kernel ids in the order of kernels::kernel (cpp/purify/kernels.h:15). */
typedef enum {
  PURIFY_GB300_KERNEL_KB = 0,
  PURIFY_GB300_KERNEL_GAUSS = 1,
  PURIFY_GB300_KERNEL_BOX = 2,
  PURIFY_GB300_KERNEL_PSWF = 3,
  PURIFY_GB300_KERNEL_KBMIN = 4,
  PURIFY_GB300_KERNEL_GAUSS_ALT = 5
} purify_gb300_kernel;

typedef enum { PURIFY_GB300_FP32 = 0, PURIFY_GB300_FP64 = 1 } purify_gb300_precision;

typedef struct purify_gb300_operator purify_gb300_operator;

/* Everything init_degrid_operator_2d takes (operators.h:373-380), plus the
 * precision.  power_iters = 0 leaves the norm at 1 (call power_method later). */
typedef struct {
  const double *u;       /* M coordinates, grid pixels */
  const double *v;       /* M */
  const double *w;       /* M, or NULL (only read when w_term != 0) */
  const double *weights; /* M complex (c128), or NULL for all ones */
  int64_t M;
  uint32_t imsizey, imsizex;
  double oversample_ratio; /* default 2 */
  uint32_t power_iters;    /* default 100 */
  double power_tol;        /* default 1e-4 */
  int32_t kernel;          /* purify_gb300_kernel, default KB */
  uint32_t Ju, Jv;         /* default 4, 4 */
  int32_t w_term;          /* default 0 */
  uint32_t Jw;             /* default 6 */
  double cellx, celly;     /* arcsec, default 1, 1 */
  int32_t precision;       /* purify_gb300_precision */
  int32_t device;          /* CUDA device ordinal */
  /* Extension: per-row w-support (M values, Jw of each visibility) when
   * w_term != 0, or NULL to use Jw for every row as the reference does.
   * Supports Jw + J - 1 up to 32 taps per axis. */
  const int32_t *jw_rows;
} purify_gb300_create_args;

/* Fills `args` with the reference's defaults (operators.h:373-380). */
void purify_gb300_default_args(purify_gb300_create_args *args);

/* Builds S, Z, F and G (the coverage plan) on the device, then runs the power
 * method when power_iters > 0 and normalises both directions by the norm.
 * Replaces measurementoperator::init_degrid_operator_2d (operators.h:373-396). */
int purify_gb300_operator_create(const purify_gb300_create_args *args,
                                 purify_gb300_operator **out);
int purify_gb300_operator_destroy(purify_gb300_operator *op);

/* Launch and layout parameters; 0 (or -1 for fused_permute) picks the
 * default.  No counterpart in the reference (its operator has no launch
 * shapes); the autotuner searches these. */
typedef struct {
  int32_t threads;       /* CTA threads of the degrid/grid kernels, multiple of 32, <= 256
                            (0: 64 for supports J >= 6, else 128) */
  int32_t max_per_item;  /* visibilities of one base cell given to one lane (<= 65535) */
  int32_t tile;          /* uv tile edge in grid cells (<= 255) */
  int32_t fused_permute; /* 1: degrid/grid touch caller-ordered visibilities directly,
                            0: via a slot-ordered buffer and gather kernels, -1: default
                            (Phi direct; Phi^H direct for supports J >= 4, else through
                            the slot-ordered buffer, and always so with weights or with
                            the column walk) */
  int32_t cell_group;    /* base cells of a work item: 0 or 1 = one cell (the default);
                            2 = an aligned 2 x 2 cell group, a (J + 1)^2 register block;
                            3 = an aligned pair of cells of a row, a J x (J + 1) block
                            (2 and 3: complex<float>, J <= 6) */
  int32_t class_cap;     /* most items of one shared-memory bank class in a batch of 32
                            (1 .. 16), or 0 for the default */
  int32_t keep_store;    /* 1: Phi's caller-ordered output is stored at L2 evict-last
                            priority (when it fits the L2 share), for a following Phi^H */
  int32_t fft_columns;   /* column transforms of the FP32 power-of-two FFT path: 0 = the
                            library's column pass (grid height <= 2048), 1 = cuFFT's
                            strided column plan */
  int32_t grid_walk;     /* G^H of Phi^H: 1 = the column walk where it applies (tiles <= 32,
                            single-cell items, J <= 8, J <= 6 in FP64), 0 = work items */
  int32_t normal_pass;   /* G^H G of purify_gb300_normal and the power method: 1 = one
                            pass over each task where it applies (FP32, unit weights,
                            single-cell items, J <= 6), 2 = degrid then grid through the
                            slot-ordered buffer, 0 = default (one pass for J < 6); the
                            results are bit-identical */
} purify_gb300_tuning;
int purify_gb300_operator_create_tuned(const purify_gb300_create_args *args,
                                       const purify_gb300_tuning *tuning,
                                       purify_gb300_operator **out);

/* Phi x and Phi^H y on device buffers of the operator's precision (c64 for
 * FP32, c128 for FP64).  x has imsizey*imsizex values, y has M values.  The
 * work is ordered after prior work on `stream` (a cudaStream_t, 0 = legacy
 * default stream) and later work on `stream` sees the result.
 * Replaces the direct/indirect closures of operators.h:325-326,393-395. */
int purify_gb300_forward(purify_gb300_operator *op, const void *x, void *y, void *stream);
int purify_gb300_adjoint(purify_gb300_operator *op, const void *y, void *x, void *stream);

/* Same on host complex<double> vectors (the reference's Vector<t_complex>);
 * copies in and out of the device inside the call, which returns when the
 * result is in `y` / `x`.  Replaces the host_wrapper path of
 * operators_gpu.h:42-68. */
int purify_gb300_forward_host(purify_gb300_operator *op, const double *x, double *y);
int purify_gb300_adjoint_host(purify_gb300_operator *op, const double *y, double *x);

/* Phi^H Phi x on device buffers (x and out: imsizey*imsizex values; they may
 * be the same buffer), the visibilities kept in the operator's internal order
 * between the two halves.  This is the combined degridding/gridding operator
 * of operators::init_grid_degrid_operator_2d (compact_operators.h:147-174):
 * with the operator's norm from its power method it is Phi'^H Phi' /
 * ||Phi'||^2, what the reference computes with the G^H G sparse matrix
 * (pruned at 1e-7, compact_operators.h:103-116); here nothing is pruned. */
int purify_gb300_normal(purify_gb300_operator *op, const void *x, void *out, void *stream);

/* Convolution with the point-spread function, the image-domain approximation
 * of Phi^H Phi (operators::init_psf_convolve_2d, compact_operators.h:279-307):
 * psf = Phi^H Phi delta with delta at pixel (floor(imsizey/2) - 1,
 * floor(imsizex/2) - 1); apply(x) = F^-1 (F psf . F x) / ||.||^2 with the
 * unitary imsizey x imsizex FFT F (circular, no padding) and the norm from
 * power_iters power-method rounds on the unnormalised convolution. */
typedef struct purify_gb300_psf purify_gb300_psf;
int purify_gb300_psf_create(purify_gb300_operator *op, uint32_t power_iters, double power_tol,
                            purify_gb300_psf **out);
int purify_gb300_psf_apply(purify_gb300_psf *p, const void *x, void *out, void *stream);
int purify_gb300_psf_norm(const purify_gb300_psf *p, double *norm);
int purify_gb300_psf_destroy(purify_gb300_psf *p);

/* G and G^H alone on device buffers of the operator's precision: grid is
 * ftsizev*ftsizeu values (index p * ftsizeu + q), vis is M values.  Replaces
 * the closures of operators::init_gridding_matrix_2d (operators.h:123-145). */
int purify_gb300_degrid(purify_gb300_operator *op, const void *grid, void *vis, void *stream);
int purify_gb300_grid(purify_gb300_operator *op, const void *vis, void *grid, void *stream);

/* G^H that allocates nothing, for callers that may not call cudaMalloc once
 * running (all device memory handed to a pool at start-up, or a hard memory
 * cap on a shared GPU).  Same inputs, output and result as purify_gb300_grid;
 * its scratch (accumulation windows and the slot-ordered visibility buffer)
 * lives in one fixed array of PURIFY_GB300_STATIC_SCRATCH_BYTES that is part
 * of the library and stays resident on every GPU that loads it.  An operator
 * whose scratch would not fit is refused with PURIFY_GB300_INVALID_ARGUMENT
 * (purify_gb300_grid_no_alloc_bytes tells the need).  The first call on a
 * device looks up the array's address and keeps it for the life of the
 * process; make that first call before any stream capture.  The kept
 * address dies with the device's context, so cudaDeviceReset after the
 * first call is not supported (it also frees every operator's device
 * state).  Every call shares the array and leaves its contents
 * behind, so calls that overlap on the GPU (any operator, any stream) race:
 * order them.  Everything the kernels read from the array is written first
 * in the same call.  No counterpart in the reference. */
#define PURIFY_GB300_STATIC_SCRATCH_BYTES (32u << 20)
int purify_gb300_grid_no_alloc(purify_gb300_operator *op, const void *vis, void *grid,
                               void *stream);
int purify_gb300_grid_no_alloc_bytes(const purify_gb300_operator *op, int64_t *bytes);

/* Gridding correction S(j, i) as imsizey*imsizex complex<double> values
 * (row j, column i), as details::init_correction2d builds it
 * (operators.cc:101-121).  Host only. */
int purify_gb300_correction(int32_t kernel, uint32_t Ju, uint32_t Jv, uint32_t imsizey,
                            uint32_t imsizex, double oversample_ratio, double *S_out);

/* Power method on Phi'^H Phi' (the unnormalised operator) from the all-ones
 * vector; sets and returns ||Phi'|| (operators.h:390-392, sopt::power_method). */
int purify_gb300_power_method(purify_gb300_operator *op, uint32_t iters, double tol,
                              double *norm_out);
/* Sets / reads the norm both directions divide by (operators.h:185-189). */
int purify_gb300_set_norm(purify_gb300_operator *op, double norm);
int purify_gb300_get_norm(const purify_gb300_operator *op, double *norm);

/* Per-stage device timing with CUDA events recorded on the operator's own
 * stream around each stage (pad, FFT forward, degrid, grid, fold, FFT
 * inverse, crop, compact, expand).  enable != 0 starts recording and clears
 * the totals; purify_gb300_stage_times waits for the recorded work and
 * returns the total milliseconds and launch count of each stage
 * (PURIFY_GB300_STAGES entries each).  No
 * counterpart in the reference (its benchmarks time whole applies with
 * std::chrono, cpp/benchmarks/measurement_operator.cc:124-125). */
#define PURIFY_GB300_STAGES 9
int purify_gb300_stage_timing(purify_gb300_operator *op, int enable);
int purify_gb300_stage_times(purify_gb300_operator *op, double *total_ms, int64_t *launches);

typedef struct {
  int64_t M;
  uint32_t imsizey, imsizex, ftsizev, ftsizeu;
  uint32_t Ju, Jv;
  int32_t precision;
  int32_t kernel;
  int32_t w_term;
  int64_t nnz;             /* non-zeros of G (taps) */
  int64_t occupied_cells;  /* distinct base cells of the coverage */
  int64_t work_items;      /* lane work items incl. padding */
  int64_t tasks;           /* CTA tasks per apply */
  int64_t device_bytes;    /* device memory held by the operator */
  double kernel_fit_error; /* max |poly - kernel| of the tap weights (abs) */
  double norm;
  int64_t slots;           /* per-slot coverage entries (M plus null slots; M with w_term) */
  int64_t window_cells;    /* grid cells of one task's accumulation window */
  int64_t factor_values;   /* w_term: complex row-factor values stored (0 otherwise) */
  int64_t cell_group;      /* work-item shape: 1 one cell, 2 a 2 x 2 group, 3 a pair of a row */
  int64_t walk_tasks;      /* tasks of the column-walk G^H of Phi^H (0: it uses work items) */
  int64_t walk_steps;      /* column steps of the walk: sum over its columns of the fullest row */
} purify_gb300_info;
int purify_gb300_operator_info(const purify_gb300_operator *op, purify_gb300_info *info);

/* utilities::set_cell_size + uv_scale (utilities.cc:208-278): wavelengths ->
 * grid pixels for a ftsizeu x ftsizev grid; cell sizes in arcsec, 0 derives
 * them from max |u|, |v| as the reference does. */
int purify_gb300_lambda_to_pixels(const double *u, const double *v, int64_t M, double cellx,
                                  double celly, uint32_t ftsizeu, uint32_t ftsizev,
                                  double *u_out, double *v_out);

/* Units of visibility coordinates, in the order of utilities::vis_units
 * (cpp/purify/utilities.h:14). */
typedef enum {
  PURIFY_GB300_UNITS_LAMBDA = 0,  /* wavelengths */
  PURIFY_GB300_UNITS_RADIANS = 1, /* units of 2 pi across the grid */
  PURIFY_GB300_UNITS_PIXELS = 2   /* grid pixels */
} purify_gb300_units;
/* The unit pipeline of the vis_params overload of init_degrid_operator_2d
 * (operators.h:405-410): wavelengths go through set_cell_size (to radians)
 * and then uv_scale (to pixels, utilities.cc:258-278); radians go through
 * uv_scale alone; pixels are copied unchanged.  Cell sizes in arcsec, used
 * for wavelengths only (0 derives them from max |u|, |v|).  An unknown unit
 * is PURIFY_GB300_INVALID_ARGUMENT. */
int purify_gb300_uv_to_pixels(const double *u, const double *v, int64_t M, int32_t units,
                              double cellx, double celly, uint32_t ftsizeu, uint32_t ftsizev,
                              double *u_out, double *v_out);

/* ---- Host-side introspection (no GPU work) --------------------------------
 * The coverage plan the operator uploads.  Visibilities are sorted by uv tile
 * and base cell and grouped into work items (one base cell, up to 16
 * visibilities); 32 items with distinct base cells form a batch, and a batch
 * owns 32 * kmax "slots" (kmax = its longest item) with lane l's k-th
 * visibility in slot base + 32 k + l.  No counterpart in the reference (its G
 * is an explicit CSR matrix, operators.cc:8-46); exposed so host logic can be
 * tested without a GPU. */
typedef struct purify_gb300_plan purify_gb300_plan;
int purify_gb300_plan_create(const double *u, const double *v, const double *weights, int64_t M,
                             uint32_t ftsizeu, uint32_t ftsizev, uint32_t J,
                             purify_gb300_plan **out);
/* The same plan with work items of several base cells (group 1, 2 or 3;
 * with 2 an item is an aligned 2 x 2 cell group of its tile, with 3 an
 * aligned pair of cells of a row; lp and lq are its anchor and each fraction
 * carries the visibility's cell in the group as its integer part: frac =
 * t + d, d in {0, 1}). */
int purify_gb300_plan_create_grouped(const double *u, const double *v, const double *weights,
                                     int64_t M, uint32_t ftsizeu, uint32_t ftsizev, uint32_t J,
                                     int32_t group, purify_gb300_plan **out);
/* sizes[0..10] = M, slots, batches, tasks, tiles along u, tiles along v,
 * window rows, window columns, unit-weight flag, group, window row stride. */
int purify_gb300_plan_sizes(const purify_gb300_plan *plan, int64_t *sizes);
/* Per slot: frac (2 doubles t_u, t_v), weight (2 doubles, the weight times the
 * phase sign (-1)^(k_u + k_v); 0 for null slots), slot_user (caller index or
 * -1).  Per visibility: user_slot.  Per batch: batches (2 int32: first slot,
 * kmax) and lane_code (32 int32: lp | lq << 8 | count << 16).  Per task:
 * tasks (8 int32: P, Q, H, W, batch_begin, batch_end, tile, 0).  tile_tasks:
 * tiles + 1; tu_start: tiles_u + 1; tv_start: tiles_v + 1.  Any pointer may
 * be NULL. */
int purify_gb300_plan_export(const purify_gb300_plan *plan, double *frac, double *weight,
                             int32_t *slot_user, int32_t *user_slot, int32_t *batches,
                             int32_t *lane_code, int32_t *tasks, int32_t *tile_tasks,
                             int32_t *tu_start, int32_t *tv_start);
int purify_gb300_plan_destroy(purify_gb300_plan *plan);
/* The column-walk plan of G^H that Phi^H uses (tiles of 32, J x J taps):
 * one task per occupied tile; lanes are the tile's rows, and a warp walks its
 * base-cell columns in order.  Slots (S = M, no null slots) follow the walk:
 * per task, per column q, per k = 0, 1, ...: the k-th visibility of every row
 * with more than k in that column, rows ascending.  sizes[0..7] = M, tasks,
 * tiles along u, tiles along v, window rows, window columns, window row
 * stride (odd), column steps (sum over columns of the fullest row). */
typedef struct purify_gb300_walk_plan purify_gb300_walk_plan;
int purify_gb300_walk_plan_create(const double *u, const double *v, int64_t M, uint32_t ftsizeu,
                                  uint32_t ftsizev, uint32_t J, purify_gb300_walk_plan **out);
int purify_gb300_walk_plan_sizes(const purify_gb300_walk_plan *plan, int64_t *sizes);
/* Per slot: frac (2 doubles: t_u with the phase sign (-1)^(k_u + k_v), t_v)
 * and slot_user (caller index).  Per task: counts (32 columns x 32 rows),
 * colstart (33: first slot of each column, then the end), tasks (8 int32:
 * P, Q, H, W, 0, 0, tile, 0); task_order (launch order); tile_tasks (tiles +
 * 1).  Any pointer may be NULL. */
int purify_gb300_walk_plan_export(const purify_gb300_walk_plan *plan, double *frac,
                                  int32_t *slot_user, int32_t *counts, int32_t *colstart,
                                  int32_t *tasks, int32_t *task_order, int32_t *tile_tasks);
int purify_gb300_walk_plan_destroy(purify_gb300_walk_plan *plan);
/* Tap weights as the device evaluates them: for each t in [0, 1) the J values
 * (-1)^j kernel(t + J/2 - 1 - j), j = 0..J-1, from the fitted polynomials
 * evaluated in the precision's arithmetic (out: n * J doubles).  Returns the
 * fit's max deviation in *fit_error when non-null.  kernels.cc:7-230. */
int purify_gb300_kernel_taps(int32_t kernel, uint32_t J, double oversample_ratio,
                             int32_t precision, const double *t, int64_t n, double *out,
                             double *fit_error);

/* One w-projection row as the device rebuilds it from its stored factors:
 * the S x S values (S = Jw + J - 1, row-major, v then u) of the gridding
 * matrix row of a visibility at (u, v) pixels with w - mean(w) = w_centered,
 * weight 1, phase included (out: 2 S S doubles).  Host only; operators.cc:49-99,
 * projection_kernels.cc:59-85. */
int purify_gb300_wrow_taps(double u, double v, double w_centered, uint32_t Jw, uint32_t J,
                           int32_t kernel, double oversample_ratio, uint32_t imsizey,
                           uint32_t imsizex, double cellx, double celly, double *out);

/* ---- Multi-channel batch -------------------------------------------------
 * Many operators (frequency channels or snapshots, each with its own coverage,
 * visibility count and image size; one kernel, support and oversampling)
 * applied together.  A step over all channels is a fixed set of grouped
 * launches -- one degrid and one grid launch over every channel's tasks,
 * element-wise kernels over all channels, one batched cuFFT per grid size --
 * recorded once into a CUDA graph and replayed.  Each channel's result is
 * that of a single operator built from its coverage (within the precision's
 * rounding).  The reference applies such a set one operator after another
 * (init_combine_operators / init_super_operator, operators.h:513-578). */
typedef struct purify_gb300_batch purify_gb300_batch;
typedef struct {
  const double *u, *v;    /* M coordinates in grid pixels */
  const double *weights;  /* M complex<double>, or NULL for ones */
  int64_t M;
  uint32_t imsizey, imsizex;
} purify_gb300_channel;
/* Tile edge and CTA sizes of a batch.  No counterpart in the reference. */
typedef struct {
  int32_t tile;            /* uv tile edge in grid cells */
  int32_t max_per_item;    /* visibilities of one base cell given to one lane */
  int32_t degrid_threads;  /* CTA threads of the grouped degrid launch */
  int32_t grid_threads;    /* CTA threads of the grouped grid launch */
  int32_t cell_group;      /* work-item shape: 1, or 2 (2 x 2) / 3 (row pairs) for FP32, J <= 6 */
  int32_t fft_columns;     /* column transforms of FP32 power-of-two grids: 0 = the library's
                              column pass (grid height <= 2048), 1 = cuFFT's strided plan */
} purify_gb300_batch_tuning;
/* Builds the batch (plans every channel, uploads the coverage state).  With
 * tuning == NULL the autotuner picks the tile edge and CTA sizes by timing
 * candidates on the GPU (a sample of up to 8 channels; cached per process).
 * Norms start at 1; see purify_gb300_batch_power_method. */
int purify_gb300_batch_create(const purify_gb300_channel *channels, int32_t nch,
                              double oversample_ratio, int32_t kernel, uint32_t J,
                              int32_t precision, int32_t device,
                              const purify_gb300_batch_tuning *tuning, purify_gb300_batch **out);
int purify_gb300_batch_destroy(purify_gb300_batch *b);
/* The tuning the batch runs with (the autotuner's pick when it chose). */
int purify_gb300_batch_get_tuning(const purify_gb300_batch *b, purify_gb300_batch_tuning *t);
/* Binds per-channel device buffers (arrays of nch pointers; complex of the
 * batch's precision): x_in (imsizey*imsizex, forward input), vis (M, forward
 * output and adjoint input), x_out (imsizey*imsizex, adjoint output).  Any
 * array may be NULL when the directions that use it are not applied.  The
 * pointers live in device tables read by the recorded graph, so rebinding
 * needs no new recording.  Ordered on `stream` like an apply. */
int purify_gb300_batch_bind(purify_gb300_batch *b, const void *const *x_in, void *const *vis,
                            void *const *x_out, void *stream);
/* One step over every channel: directions 1 = Phi (x_in -> vis), 2 = Phi^H
 * (vis -> x_out), 3 = both in turn (x_out = Phi^H Phi x_in).  Ordered after
 * prior work on `stream`; later work on `stream` sees the results. */
int purify_gb300_batch_apply(purify_gb300_batch *b, int32_t directions, void *stream);
/* Power method of every channel together, each channel with the
 * single-operator rule (operators.h:390-391); sets the per-channel norms and
 * writes them to norms (nch doubles) when not NULL.  Synchronous. */
int purify_gb300_batch_power_method(purify_gb300_batch *b, uint32_t iters, double tol,
                                    double *norms);
int purify_gb300_batch_set_norms(purify_gb300_batch *b, const double *norms);
int purify_gb300_batch_get_norms(const purify_gb300_batch *b, double *norms);
typedef struct {
  int32_t channels, size_groups;
  int64_t visibilities, pixels, tasks, device_bytes;
} purify_gb300_batch_info;
int purify_gb300_batch_info_get(const purify_gb300_batch *b, purify_gb300_batch_info *info);
/* Average device milliseconds of one replay over `reps` replays (after two
 * untimed ones) on the batch's own scratch buffers: what = 1, 2, 3 as in
 * purify_gb300_batch_apply, 8 = the grouped degrid launch alone, 16 = the
 * grouped grid launch alone.  The binding is kept.  No counterpart in the
 * reference; used by the autotuner and the benchmark. */
int purify_gb300_batch_time(purify_gb300_batch *b, int32_t what, uint32_t reps, double *ms);

/* ---- Solver-side consumer ---------------------------------------------------
 * Forward-backward (proximal gradient) iterations of
 *   min_x 1/2 ||y - Phi x||^2 + gamma ||x||_1  (x real and >= 0 optionally)
 * on the device: b = Phi^H y, then per iteration
 *   x <- soft_{step gamma}(x - step (Phi^H Phi x - b))
 * through purify_gb300_normal, followed by the reference's step-size update
 * of gamma (cpp/purify/update_factory.h:46-54: gamma' = update_scale
 * max |Re x|, taken when |gamma - gamma'| > update_tol during the first
 * update_iters iterations).  gamma starts at gamma_scale max |Phi^H y|, as
 * the reference's PADMM factory sets it (cpp/purify/algorithm_factory.h:
 * 73-76).  This stands in for the reference's solvers (sopt's proximal ADMM,
 * absent here) as the caller that applies Phi^H Phi many times per solve. */
typedef struct {
  uint32_t iterations;
  double step;              /* gradient step; 1 for a normalised operator */
  double gamma_scale;       /* default 1e-3 */
  double update_scale;      /* default 1e-3 (step_size_scale) */
  double update_tol;        /* default 1e-3 */
  uint32_t update_iters;    /* default 0: gamma keeps its start value */
  int32_t real_constraint;  /* default 1 */
  int32_t positive_constraint; /* default 1 */
} purify_gb300_fb_params;
void purify_gb300_fb_default_params(purify_gb300_fb_params *p);
/* y: M device values, x: imsizey * imsizex device values (start on entry,
 * solution on exit), both of the operator's precision; gammas: host array of
 * `iterations` doubles receiving the gamma each iteration used, or NULL.
 * Ordered after `stream`; returns when the solve has finished. */
int purify_gb300_forward_backward(purify_gb300_operator *op, const void *y, void *x,
                                  const purify_gb300_fb_params *params, double *gammas,
                                  void *stream);

/* ---- Request server ------------------------------------------------------
 * Forward, adjoint and operator-norm requests on coverages kept resident on
 * the device, admitted by an HBM budget and run concurrently: each admitted
 * request gets its own workspace (grids, task windows, I/O vectors) from a
 * stream-ordered memory pool and one of `slots` CUDA streams, so requests
 * that arrive while others run are admitted as streams and memory free up
 * and their kernels overlap on the GPU.  A request shares no scratch with
 * another, so its result is the same alone and in a mix.  No counterpart in
 * the reference (its operators are applied by one solver at a time). */
typedef struct purify_gb300_server purify_gb300_server;
typedef struct {
  int32_t device;
  int32_t slots;             /* requests in flight at most (1..64) */
  int64_t hbm_budget_bytes;  /* device bytes of the requests in flight */
  int32_t norm_slots;        /* slots norm requests may hold (0: slots / 4, at least 1); they
                                run on the lowest stream priority, other requests on the
                                highest, so short requests are scheduled first */
} purify_gb300_server_config;
int purify_gb300_server_create(const purify_gb300_server_config *cfg, purify_gb300_server **out);
/* Destroys after the requests already submitted have run. */
int purify_gb300_server_destroy(purify_gb300_server *s);
/* Builds a resident coverage from operator arguments (power_iters > 0 sets
 * its norm) and returns its id. */
int purify_gb300_server_add_coverage(purify_gb300_server *s, const purify_gb300_create_args *args,
                                     int32_t *coverage);
#define PURIFY_GB300_REQ_FORWARD 1         /* vis_out = Phi x_in */
#define PURIFY_GB300_REQ_ADJOINT 2         /* x_out = Phi^H vis_in (dirty image) */
#define PURIFY_GB300_REQ_FORWARD_ADJOINT 3 /* vis_out = Phi x_in, x_out = Phi^H vis_out */
#define PURIFY_GB300_REQ_NORM 4            /* ||Phi'|| by iters power-method rounds */
/* Host vectors are complex<double>; inputs are copied at submit, outputs
 * written by purify_gb300_server_wait. */
typedef struct {
  int32_t coverage;
  int32_t kind;
  const double *x_in;
  const double *vis_in;
  double *vis_out;
  double *x_out;
  uint32_t iters; /* norm requests */
  double tol;     /* norm requests: the power method's stopping rule */
} purify_gb300_request;
int purify_gb300_server_submit(purify_gb300_server *s, const purify_gb300_request *rq,
                               int64_t *ticket);
typedef struct {
  int32_t status;      /* of the request: OK, REJECTED (never fits the budget), ... */
  int32_t iterations;  /* norm requests: rounds until the stopping rule held */
  double norm;
  double queue_ms, run_ms, latency_ms; /* submit->admit, admit->done, submit->done */
  int64_t device_bytes;
} purify_gb300_result;
/* Waits up to timeout_s seconds (< 0: no limit); returns
 * PURIFY_GB300_TIMEOUT if the request is still running, else copies its
 * outputs, fills *out and forgets the ticket. */
int purify_gb300_server_wait(purify_gb300_server *s, int64_t ticket, double timeout_s,
                             purify_gb300_result *out);
/* Device bytes a request would hold while in flight. */
int purify_gb300_server_request_bytes(const purify_gb300_server *s, const purify_gb300_request *rq,
                                      int64_t *bytes);
typedef struct {
  int64_t submitted, completed, rejected, failed;
  int64_t inflight_peak, bytes_peak, bytes_budget;
  double latency_p50_ms, latency_p99_ms, latency_mean_ms; /* completed requests */
  double visibility_passes; /* sum of M x (G and G^H passes) of completed requests */
} purify_gb300_server_stats;
int purify_gb300_server_get_stats(const purify_gb300_server *s, purify_gb300_server_stats *out);

/* ---- Coverage ingest -------------------------------------------------------
 * The reference's .vis text format (utilities::read_visibility,
 * utilities.cc:140-188): per row u v [w] re(V) im(V) sigma separated by white
 * space, nan / inf accepted; v is negated on reading (utilities.cc:178) and
 * the weight is 1 / sigma.  purify_gb300_vis_file_rows counts the rows;
 * purify_gb300_read_visibility fills u, v, w (NULL allowed when !w_term),
 * vis and weights (complex<double>, rows values each).  Host only. */
int purify_gb300_vis_file_rows(const char *path, int64_t *rows);
int purify_gb300_read_visibility(const char *path, int32_t w_term, int64_t rows, double *u,
                                 double *v, double *w, double *vis, double *weights);
/* utilities::init_weights (utilities.cc:569-608): none (all 1), natural and
 * whiten (the weights unchanged), uniform (w / sqrt(n)) and robust
 * (w / sqrt(1 + s n), s = sum w^2 / sum n^2 * 25 * 10^(-2R)), with n the
 * number of visibilities in the ftsizev x ftsizeu cell of floor(u / oversample),
 * floor(v / oversample) (periodic).  The histogram and the sums run on the
 * device (integer atomics, fixed-order FP64 reductions); host buffers. */
#define PURIFY_GB300_WEIGHT_NONE 0
#define PURIFY_GB300_WEIGHT_NATURAL 1
#define PURIFY_GB300_WEIGHT_WHITEN 2
#define PURIFY_GB300_WEIGHT_UNIFORM 3
#define PURIFY_GB300_WEIGHT_ROBUST 4
int purify_gb300_init_weights(const double *u, const double *v, const double *weights, int64_t M,
                              double oversample_factor, int32_t weighting, double R,
                              uint32_t ftsizeu, uint32_t ftsizev, int32_t device, double *out);

/* Message of the last failing call on this thread ("" when none). */
const char *purify_gb300_last_error(void);
/* Library version string. */
const char *purify_gb300_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PURIFY_GB300_H */
