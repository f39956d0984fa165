"""Python mirror of the GB300 measurement operator's C ABI.

``MeasurementOperator`` takes the arguments of the reference's
``measurementoperator::init_degrid_operator_2d`` (cpp/purify/operators.h:373-380)
with u, v in grid pixels, and applies Phi / Phi^H through
``libpurify_gb300.so``:

* ``forward(x)`` / ``adjoint(y)`` on torch CUDA tensors of the operator's
  complex dtype (complex64 for FP32, complex128 for FP64) run on the device
  and return device tensors;
* ``forward(x)`` / ``adjoint(y)`` on numpy arrays go through the host entry
  points (complex128 in and out, copies inside the call), like the
  reference's ``Vector<t_complex>`` closures.

There is no CPU fallback: if the native library cannot be loaded every call
raises.
"""
import ctypes
import os

import numpy as np

from ._build import LIB_PATH, build  # noqa: F401

KERNELS = {"kb": 0, "gauss": 1, "box": 2, "pswf": 3, "kbmin": 4, "gauss_alt": 5}
PRECISIONS = {"fp32": 0, "fp64": 1}
STATUS = {
    0: "OK", 1: "INVALID_ARGUMENT", 2: "UNSUPPORTED", 3: "CUDA_ERROR", 4: "OUT_OF_MEMORY",
    5: "NORM_NOT_POSITIVE", 6: "REJECTED", 7: "TIMEOUT", 8: "INTERNAL",
}


class PurifyError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


class CreateArgs(ctypes.Structure):
    _fields_ = [
        ("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_void_p),
        ("weights", ctypes.c_void_p), ("M", ctypes.c_int64),
        ("imsizey", ctypes.c_uint32), ("imsizex", ctypes.c_uint32),
        ("oversample_ratio", ctypes.c_double), ("power_iters", ctypes.c_uint32),
        ("power_tol", ctypes.c_double), ("kernel", ctypes.c_int32),
        ("Ju", ctypes.c_uint32), ("Jv", ctypes.c_uint32), ("w_term", ctypes.c_int32),
        ("Jw", ctypes.c_uint32), ("cellx", ctypes.c_double), ("celly", ctypes.c_double),
        ("precision", ctypes.c_int32), ("device", ctypes.c_int32), ("jw_rows", ctypes.c_void_p),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [("threads", ctypes.c_int32), ("max_per_item", ctypes.c_int32),
                ("tile", ctypes.c_int32), ("fused_permute", ctypes.c_int32),
                ("cell_group", ctypes.c_int32), ("class_cap", ctypes.c_int32),
                ("keep_store", ctypes.c_int32), ("fft_columns", ctypes.c_int32),
                ("grid_walk", ctypes.c_int32), ("normal_pass", ctypes.c_int32)]


class Info(ctypes.Structure):
    _fields_ = [
        ("M", ctypes.c_int64), ("imsizey", ctypes.c_uint32), ("imsizex", ctypes.c_uint32),
        ("ftsizev", ctypes.c_uint32), ("ftsizeu", ctypes.c_uint32), ("Ju", ctypes.c_uint32),
        ("Jv", ctypes.c_uint32), ("precision", ctypes.c_int32), ("kernel", ctypes.c_int32),
        ("w_term", ctypes.c_int32), ("nnz", ctypes.c_int64), ("occupied_cells", ctypes.c_int64),
        ("work_items", ctypes.c_int64), ("tasks", ctypes.c_int64),
        ("device_bytes", ctypes.c_int64), ("kernel_fit_error", ctypes.c_double),
        ("norm", ctypes.c_double), ("slots", ctypes.c_int64), ("window_cells", ctypes.c_int64),
        ("factor_values", ctypes.c_int64), ("cell_group", ctypes.c_int64),
        ("walk_tasks", ctypes.c_int64), ("walk_steps", ctypes.c_int64),
    ]


class Channel(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("weights", ctypes.c_void_p),
                ("M", ctypes.c_int64), ("imsizey", ctypes.c_uint32), ("imsizex", ctypes.c_uint32)]


class FbParams(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("step", ctypes.c_double),
                ("gamma_scale", ctypes.c_double), ("update_scale", ctypes.c_double),
                ("update_tol", ctypes.c_double), ("update_iters", ctypes.c_uint32),
                ("real_constraint", ctypes.c_int32), ("positive_constraint", ctypes.c_int32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("tile", ctypes.c_int32), ("max_per_item", ctypes.c_int32),
                ("degrid_threads", ctypes.c_int32), ("grid_threads", ctypes.c_int32),
                ("cell_group", ctypes.c_int32), ("fft_columns", ctypes.c_int32)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("channels", ctypes.c_int32), ("size_groups", ctypes.c_int32),
                ("visibilities", ctypes.c_int64), ("pixels", ctypes.c_int64),
                ("tasks", ctypes.c_int64), ("device_bytes", ctypes.c_int64)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_int32),
                ("hbm_budget_bytes", ctypes.c_int64), ("norm_slots", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("coverage", ctypes.c_int32), ("kind", ctypes.c_int32), ("x_in", ctypes.c_void_p),
                ("vis_in", ctypes.c_void_p), ("vis_out", ctypes.c_void_p),
                ("x_out", ctypes.c_void_p), ("iters", ctypes.c_uint32), ("tol", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("norm", ctypes.c_double), ("queue_ms", ctypes.c_double),
                ("run_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("device_bytes", ctypes.c_int64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("rejected", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("inflight_peak", ctypes.c_int64), ("bytes_peak", ctypes.c_int64),
                ("bytes_budget", ctypes.c_int64), ("latency_p50_ms", ctypes.c_double),
                ("latency_p99_ms", ctypes.c_double), ("latency_mean_ms", ctypes.c_double),
                ("visibility_passes", ctypes.c_double)]


REQUEST_KINDS = {"forward": 1, "adjoint": 2, "forward_adjoint": 3, "norm": 4}


# Every symbol include/purify_gb300.h declares (checked by the CPU tests).
EXPORTS = [
    "purify_gb300_default_args", "purify_gb300_operator_create", "purify_gb300_operator_destroy",
    "purify_gb300_forward", "purify_gb300_adjoint", "purify_gb300_forward_host",
    "purify_gb300_adjoint_host", "purify_gb300_power_method", "purify_gb300_set_norm",
    "purify_gb300_get_norm", "purify_gb300_operator_info", "purify_gb300_lambda_to_pixels",
    "purify_gb300_uv_to_pixels", "purify_gb300_fb_default_params", "purify_gb300_forward_backward",
    "purify_gb300_last_error", "purify_gb300_version", "purify_gb300_plan_create",
    "purify_gb300_plan_sizes", "purify_gb300_plan_export", "purify_gb300_plan_destroy",
    "purify_gb300_plan_create_grouped", "purify_gb300_walk_plan_create",
    "purify_gb300_walk_plan_sizes", "purify_gb300_walk_plan_export",
    "purify_gb300_walk_plan_destroy",
    "purify_gb300_kernel_taps", "purify_gb300_degrid", "purify_gb300_grid",
    "purify_gb300_correction", "purify_gb300_stage_timing", "purify_gb300_stage_times",
    "purify_gb300_operator_create_tuned", "purify_gb300_grid_no_alloc",
    "purify_gb300_grid_no_alloc_bytes", "purify_gb300_wrow_taps",
    "purify_gb300_batch_create", "purify_gb300_batch_destroy", "purify_gb300_batch_get_tuning",
    "purify_gb300_batch_bind", "purify_gb300_batch_apply", "purify_gb300_batch_power_method",
    "purify_gb300_batch_set_norms", "purify_gb300_batch_get_norms", "purify_gb300_batch_info_get",
    "purify_gb300_batch_time",
    "purify_gb300_server_create", "purify_gb300_server_destroy", "purify_gb300_server_add_coverage",
    "purify_gb300_server_submit", "purify_gb300_server_wait", "purify_gb300_server_request_bytes",
    "purify_gb300_server_get_stats", "purify_gb300_normal", "purify_gb300_psf_create",
    "purify_gb300_psf_apply", "purify_gb300_psf_norm", "purify_gb300_psf_destroy",
    "purify_gb300_vis_file_rows", "purify_gb300_read_visibility", "purify_gb300_init_weights",
]
STAGES = ["pad", "fft_forward", "degrid", "grid", "fold", "fft_inverse", "crop", "compact",
          "expand"]

_lib = None


def load(path=None):
    """Loads (building first if absent) and returns the ctypes library."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    vp, P = ctypes.c_void_p, ctypes.POINTER
    L.purify_gb300_last_error.restype = ctypes.c_char_p
    L.purify_gb300_version.restype = ctypes.c_char_p
    L.purify_gb300_default_args.argtypes = [P(CreateArgs)]
    L.purify_gb300_default_args.restype = None
    L.purify_gb300_operator_create.argtypes = [P(CreateArgs), P(vp)]
    L.purify_gb300_operator_destroy.argtypes = [vp]
    L.purify_gb300_operator_create_tuned.argtypes = [P(CreateArgs), P(Tuning), P(vp)]
    for f in (L.purify_gb300_forward, L.purify_gb300_adjoint):
        f.argtypes = [vp, vp, vp, vp]
    for f in (L.purify_gb300_forward_host, L.purify_gb300_adjoint_host):
        f.argtypes = [vp, vp, vp]
    L.purify_gb300_power_method.argtypes = [vp, ctypes.c_uint32, ctypes.c_double,
                                            P(ctypes.c_double)]
    L.purify_gb300_set_norm.argtypes = [vp, ctypes.c_double]
    L.purify_gb300_get_norm.argtypes = [vp, P(ctypes.c_double)]
    L.purify_gb300_operator_info.argtypes = [vp, P(Info)]
    L.purify_gb300_lambda_to_pixels.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_uint32,
                                                ctypes.c_uint32, vp, vp]
    L.purify_gb300_fb_default_params.argtypes = [P(FbParams)]
    L.purify_gb300_fb_default_params.restype = None
    L.purify_gb300_forward_backward.argtypes = [vp, vp, vp, P(FbParams), vp, vp]
    L.purify_gb300_uv_to_pixels.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                            ctypes.c_uint32, vp, vp]
    L.purify_gb300_plan_create.argtypes = [vp, vp, vp, ctypes.c_int64, ctypes.c_uint32,
                                           ctypes.c_uint32, ctypes.c_uint32, P(vp)]
    L.purify_gb300_plan_create_grouped.argtypes = [vp, vp, vp, ctypes.c_int64, ctypes.c_uint32,
                                                   ctypes.c_uint32, ctypes.c_uint32,
                                                   ctypes.c_int32, P(vp)]
    L.purify_gb300_plan_sizes.argtypes = [vp, vp]
    L.purify_gb300_plan_export.argtypes = [vp] + [vp] * 10
    L.purify_gb300_plan_destroy.argtypes = [vp]
    L.purify_gb300_walk_plan_create.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_uint32,
                                                ctypes.c_uint32, ctypes.c_uint32, P(vp)]
    L.purify_gb300_walk_plan_sizes.argtypes = [vp, vp]
    L.purify_gb300_walk_plan_export.argtypes = [vp] + [vp] * 7
    L.purify_gb300_walk_plan_destroy.argtypes = [vp]
    L.purify_gb300_kernel_taps.argtypes = [ctypes.c_int32, ctypes.c_uint32, ctypes.c_double,
                                           ctypes.c_int32, vp, ctypes.c_int64, vp,
                                           P(ctypes.c_double)]
    for f in (L.purify_gb300_degrid, L.purify_gb300_grid):
        f.argtypes = [vp, vp, vp, vp]
    L.purify_gb300_correction.argtypes = [ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, vp]
    L.purify_gb300_grid_no_alloc.argtypes = [vp, vp, vp, vp]
    L.purify_gb300_grid_no_alloc_bytes.argtypes = [vp, P(ctypes.c_int64)]
    L.purify_gb300_wrow_taps.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
                                         ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_double, ctypes.c_double, vp]
    L.purify_gb300_stage_timing.argtypes = [vp, ctypes.c_int]
    L.purify_gb300_stage_times.argtypes = [vp, vp, vp]
    L.purify_gb300_batch_create.argtypes = [P(Channel), ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_int32, ctypes.c_uint32, ctypes.c_int32,
                                            ctypes.c_int32, P(BatchTuning), P(vp)]
    L.purify_gb300_batch_destroy.argtypes = [vp]
    L.purify_gb300_batch_get_tuning.argtypes = [vp, P(BatchTuning)]
    L.purify_gb300_batch_bind.argtypes = [vp, vp, vp, vp, vp]
    L.purify_gb300_batch_apply.argtypes = [vp, ctypes.c_int32, vp]
    L.purify_gb300_batch_power_method.argtypes = [vp, ctypes.c_uint32, ctypes.c_double, vp]
    L.purify_gb300_batch_set_norms.argtypes = [vp, vp]
    L.purify_gb300_batch_get_norms.argtypes = [vp, vp]
    L.purify_gb300_batch_info_get.argtypes = [vp, P(BatchInfo)]
    L.purify_gb300_batch_time.argtypes = [vp, ctypes.c_int32, ctypes.c_uint32,
                                          P(ctypes.c_double)]
    L.purify_gb300_server_create.argtypes = [P(ServerConfig), P(vp)]
    L.purify_gb300_server_destroy.argtypes = [vp]
    L.purify_gb300_server_add_coverage.argtypes = [vp, P(CreateArgs), P(ctypes.c_int32)]
    L.purify_gb300_server_submit.argtypes = [vp, P(Request), P(ctypes.c_int64)]
    L.purify_gb300_server_wait.argtypes = [vp, ctypes.c_int64, ctypes.c_double, P(Result)]
    L.purify_gb300_server_request_bytes.argtypes = [vp, P(Request), P(ctypes.c_int64)]
    L.purify_gb300_server_get_stats.argtypes = [vp, P(ServerStats)]
    L.purify_gb300_normal.argtypes = [vp, vp, vp, vp]
    L.purify_gb300_psf_create.argtypes = [vp, ctypes.c_uint32, ctypes.c_double, P(vp)]
    L.purify_gb300_psf_apply.argtypes = [vp, vp, vp, vp]
    L.purify_gb300_psf_norm.argtypes = [vp, P(ctypes.c_double)]
    L.purify_gb300_psf_destroy.argtypes = [vp]
    L.purify_gb300_vis_file_rows.argtypes = [ctypes.c_char_p, P(ctypes.c_int64)]
    L.purify_gb300_read_visibility.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int64,
                                               vp, vp, vp, vp, vp]
    L.purify_gb300_init_weights.argtypes = [vp, vp, vp, ctypes.c_int64, ctypes.c_double,
                                            ctypes.c_int32, ctypes.c_double, ctypes.c_uint32,
                                            ctypes.c_uint32, ctypes.c_int32, vp]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise PurifyError(rc, load().purify_gb300_last_error().decode())


def _np_ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def lambda_to_pixels(u, v, cellx, celly, ftsizeu, ftsizev):
    """Wavelengths -> grid pixels (utilities.cc:208-278)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    uo, vo = np.empty_like(u), np.empty_like(v)
    _check(load().purify_gb300_lambda_to_pixels(_np_ptr(u), _np_ptr(v), u.size, cellx, celly,
                                                ftsizeu, ftsizev, _np_ptr(uo), _np_ptr(vo)))
    return uo, vo


UNITS = {"lambda": 0, "radians": 1, "pixels": 2}


def uv_to_pixels(u, v, units, cellx, celly, ftsizeu, ftsizev):
    """Coordinates in `units` ("lambda", "radians" or "pixels") -> grid pixels,
    the unit pipeline of the vis_params overload (operators.h:405-410)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    uo, vo = np.empty_like(u), np.empty_like(v)
    _check(load().purify_gb300_uv_to_pixels(_np_ptr(u), _np_ptr(v), u.size,
                                            UNITS.get(units, units), cellx, celly, ftsizeu,
                                            ftsizev, _np_ptr(uo), _np_ptr(vo)))
    return uo, vo


def correction(kernel, Ju, Jv, imsizey, imsizex, oversample_ratio=2.0):
    """S(j, i) of details::init_correction2d as an (imsizey, imsizex) array."""
    out = np.empty(int(imsizey) * int(imsizex), dtype=np.complex128)
    _check(load().purify_gb300_correction(KERNELS[kernel], int(Ju), int(Jv), int(imsizey),
                                          int(imsizex), float(oversample_ratio), _np_ptr(out)))
    return out.reshape(int(imsizey), int(imsizex))


def kernel_taps(kernel, J, t, oversample_ratio=2.0, precision="fp32"):
    """Tap weights as the device computes them: array (len(t), J) and the
    fit's max deviation (see purify_gb300_kernel_taps)."""
    t = np.ascontiguousarray(t, dtype=np.float64).ravel()
    out = np.empty((t.size, int(J)), dtype=np.float64)
    err = ctypes.c_double()
    _check(load().purify_gb300_kernel_taps(KERNELS[kernel], int(J), float(oversample_ratio),
                                           PRECISIONS[precision], _np_ptr(t), t.size,
                                           _np_ptr(out), ctypes.byref(err)))
    return out, err.value


def wrow_taps(u, v, w_centered, Jw, J, kernel="kb", oversample_ratio=2.0, imsizey=64,
              imsizex=64, cellx=1.0, celly=1.0):
    """One w-projection gridding-matrix row (S x S, phase included, weight 1)
    as the device rebuilds it from its factors (purify_gb300_wrow_taps)."""
    S = int(Jw) + int(J) - 1
    out = np.empty(S * S, dtype=np.complex128)
    _check(load().purify_gb300_wrow_taps(float(u), float(v), float(w_centered), int(Jw), int(J),
                                         KERNELS[kernel], float(oversample_ratio), int(imsizey),
                                         int(imsizex), float(cellx), float(celly), _np_ptr(out)))
    return out.reshape(S, S)


class CoveragePlan:
    """Host-side copy of the coverage plan (purify_gb300_plan_*)."""

    def __init__(self, u, v, ftsizeu, ftsizev, J, weights=None, group=1):
        L = load()
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        wt = None if weights is None else np.ascontiguousarray(weights, dtype=np.complex128)
        h = ctypes.c_void_p()
        _check(L.purify_gb300_plan_create_grouped(_np_ptr(u), _np_ptr(v), _np_ptr(wt), u.size,
                                                  int(ftsizeu), int(ftsizev), int(J), int(group),
                                                  ctypes.byref(h)))
        try:
            sz = np.zeros(11, dtype=np.int64)
            _check(L.purify_gb300_plan_sizes(h, _np_ptr(sz)))
            M, S, nb, nt, ntu, ntv, wr, wc, unit, grp, ws = (int(s) for s in sz)
            self.frac = np.empty((S, 2))
            self.weight = np.empty(S, dtype=np.complex128)
            self.slot_user = np.empty(S, dtype=np.int32)
            self.user_slot = np.empty(M, dtype=np.int32)
            self.batches = np.empty((nb, 2), dtype=np.int32)
            self.lane_code = np.empty((nb, 32), dtype=np.int32)
            self.tasks = np.empty((nt, 8), dtype=np.int32)
            self.tile_tasks = np.empty(ntu * ntv + 1, dtype=np.int32)
            self.tu_start = np.empty(ntu + 1, dtype=np.int32)
            self.tv_start = np.empty(ntv + 1, dtype=np.int32)
            _check(L.purify_gb300_plan_export(
                h, _np_ptr(self.frac), _np_ptr(self.weight), _np_ptr(self.slot_user),
                _np_ptr(self.user_slot), _np_ptr(self.batches), _np_ptr(self.lane_code),
                _np_ptr(self.tasks), _np_ptr(self.tile_tasks), _np_ptr(self.tu_start),
                _np_ptr(self.tv_start)))
        finally:
            L.purify_gb300_plan_destroy(h)
        self.M, self.S, self.ntu, self.ntv = M, S, ntu, ntv
        self.win_rows, self.win_cols, self.unit_weights = wr, wc, bool(unit)
        self.group, self.win_stride = grp, ws
        self.Nu, self.Nv, self.J = int(ftsizeu), int(ftsizev), int(J)


class WalkPlan:
    """Host-side copy of the column-walk plan of G^H (purify_gb300_walk_plan_*)."""

    def __init__(self, u, v, ftsizeu, ftsizev, J):
        L = load()
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        v = np.ascontiguousarray(v, dtype=np.float64).ravel()
        h = ctypes.c_void_p()
        _check(L.purify_gb300_walk_plan_create(_np_ptr(u), _np_ptr(v), u.size, int(ftsizeu),
                                               int(ftsizev), int(J), ctypes.byref(h)))
        try:
            sz = np.zeros(8, dtype=np.int64)
            _check(L.purify_gb300_walk_plan_sizes(h, _np_ptr(sz)))
            M, nt, ntu, ntv, wr, wc, ws, steps = (int(s) for s in sz)
            self.frac = np.empty((M, 2))
            self.slot_user = np.empty(M, dtype=np.int32)
            self.counts = np.empty((nt, 32, 32), dtype=np.int32)
            self.colstart = np.empty((nt, 33), dtype=np.int32)
            self.tasks = np.empty((nt, 8), dtype=np.int32)
            self.task_order = np.empty(nt, dtype=np.int32)
            self.tile_tasks = np.empty(ntu * ntv + 1, dtype=np.int32)
            _check(L.purify_gb300_walk_plan_export(
                h, _np_ptr(self.frac), _np_ptr(self.slot_user), _np_ptr(self.counts),
                _np_ptr(self.colstart), _np_ptr(self.tasks), _np_ptr(self.task_order),
                _np_ptr(self.tile_tasks)))
        finally:
            L.purify_gb300_walk_plan_destroy(h)
        self.M, self.ntu, self.ntv = M, ntu, ntv
        self.win_rows, self.win_cols, self.win_stride, self.steps = wr, wc, ws, steps
        self.Nu, self.Nv, self.J = int(ftsizeu), int(ftsizev), int(J)


def _create_args(u, v, w, weights, imsizey, imsizex, oversample_ratio, power_iters, power_tol,
                 kernel, Ju, Jv, w_term, Jw, cellx, celly, precision, device, jw_rows):
    """CreateArgs of the reference's factory arguments; returns the struct and
    the arrays it points into (keep them alive while it is used)."""
    L = load()
    u = np.ascontiguousarray(u, dtype=np.float64).ravel()
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    if v.size != u.size:
        raise PurifyError(1, "Size of u and v vectors are not the same for creating gridding matrix.")
    w = None if w is None else np.ascontiguousarray(w, dtype=np.float64).ravel()
    wt = None if weights is None else np.ascontiguousarray(weights, dtype=np.complex128).ravel()
    jw = None if jw_rows is None else np.ascontiguousarray(jw_rows, dtype=np.int32).ravel()
    a = CreateArgs()
    L.purify_gb300_default_args(ctypes.byref(a))
    a.u, a.v = _np_ptr(u), _np_ptr(v)
    a.w = _np_ptr(w)
    a.weights = _np_ptr(wt)
    a.M = u.size
    a.imsizey, a.imsizex = int(imsizey), int(imsizex)
    a.oversample_ratio = float(oversample_ratio)
    a.power_iters = int(power_iters)
    a.power_tol = float(power_tol)
    a.kernel = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
    a.Ju, a.Jv = int(Ju), int(Jv)
    a.w_term = 1 if w_term else 0
    a.Jw = int(Jw)
    a.jw_rows = _np_ptr(jw)
    a.cellx, a.celly = float(cellx), float(celly)
    a.precision = PRECISIONS[precision]
    a.device = int(device)
    return a, (u, v, w, wt, jw)


WEIGHTINGS = {"none": 0, "natural": 1, "whiten": 2, "uniform": 3, "robust": 4}


def read_visibility(path, w_term=False):
    """utilities::read_visibility (cpp/purify/utilities.cc:140-188): a .vis
    text file of u v [w] re im sigma rows; v negated, weights = 1 / sigma."""
    L = load()
    p = os.fsencode(path)
    rows = ctypes.c_int64()
    _check(L.purify_gb300_vis_file_rows(p, ctypes.byref(rows)))
    n = rows.value
    u, v, w = np.empty(n), np.empty(n), np.zeros(n)
    vis = np.empty(n, dtype=np.complex128)
    weights = np.empty(n, dtype=np.complex128)
    _check(L.purify_gb300_read_visibility(p, 1 if w_term else 0, n, _np_ptr(u), _np_ptr(v),
                                          _np_ptr(w) if w_term else None, _np_ptr(vis),
                                          _np_ptr(weights)))
    return {"u": u, "v": v, "w": w, "vis": vis, "weights": weights}


def init_weights(u, v, weights, oversample_factor, weighting, R, ftsizeu, ftsizev, device=0):
    """utilities::init_weights (cpp/purify/utilities.cc:569-608): none,
    natural, whiten, uniform or robust visibility weights."""
    u = np.ascontiguousarray(u, dtype=np.float64).ravel()
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    wt = np.ascontiguousarray(weights, dtype=np.complex128).ravel()
    if not (u.size == v.size == wt.size):
        raise PurifyError(1, "u, v and weights differ in length")
    out = np.empty_like(wt)
    _check(load().purify_gb300_init_weights(
        _np_ptr(u), _np_ptr(v), _np_ptr(wt), u.size, float(oversample_factor),
        WEIGHTINGS[weighting] if isinstance(weighting, str) else int(weighting), float(R),
        int(ftsizeu), int(ftsizev), int(device), _np_ptr(out)))
    return out


def _is_torch(x):
    return type(x).__module__.startswith("torch")


class MeasurementOperator:
    """Phi = G F Z S / ||Phi'|| on one GPU (see the module docstring)."""

    def __init__(self, u, v, w=None, weights=None, imsizey=256, imsizex=256,
                 oversample_ratio=2.0, power_iters=100, power_tol=1e-4, kernel="kb", Ju=4, Jv=4,
                 w_term=False, Jw=6, cellx=1.0, celly=1.0, precision="fp32", device=0,
                 tuning=None, jw_rows=None):
        L = load()
        a, keep = _create_args(u, v, w, weights, imsizey, imsizex, oversample_ratio, power_iters,
                               power_tol, kernel, Ju, Jv, w_term, Jw, cellx, celly, precision,
                               device, jw_rows)
        M = a.M
        h = ctypes.c_void_p()
        if tuning:
            t = Tuning(int(tuning.get("threads", 0)), int(tuning.get("max_per_item", 0)),
                       int(tuning.get("tile", 0)), int(tuning.get("fused_permute", -1)),
                       int(tuning.get("cell_group", 0)), int(tuning.get("class_cap", 0)),
                       int(tuning.get("keep_store", 0)), int(tuning.get("fft_columns", 0)),
                       int(tuning.get("grid_walk", 0)), int(tuning.get("normal_pass", 0)))
            _check(L.purify_gb300_operator_create_tuned(ctypes.byref(a), ctypes.byref(t),
                                                        ctypes.byref(h)))
        else:
            _check(L.purify_gb300_operator_create(ctypes.byref(a), ctypes.byref(h)))
        self._h = h
        self.precision = precision
        self.M = M
        self.imsizey, self.imsizex = int(imsizey), int(imsizex)
        self.device = int(device)

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().purify_gb300_operator_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def complex_dtype(self):
        import torch
        return torch.complex64 if self.precision == "fp32" else torch.complex128

    def info(self):
        i = Info()
        _check(load().purify_gb300_operator_info(self._h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in Info._fields_}

    @property
    def norm(self):
        n = ctypes.c_double()
        _check(load().purify_gb300_get_norm(self._h, ctypes.byref(n)))
        return n.value

    def set_norm(self, norm):
        _check(load().purify_gb300_set_norm(self._h, float(norm)))

    def power_method(self, iters=100, tol=1e-4):
        n = ctypes.c_double()
        _check(load().purify_gb300_power_method(self._h, int(iters), float(tol), ctypes.byref(n)))
        return n.value

    def stage_timing(self, enable=True):
        """Start (clearing totals) or stop per-stage CUDA-event timing."""
        _check(load().purify_gb300_stage_timing(self._h, 1 if enable else 0))

    def stage_times(self):
        """{stage: (total_ms, launches)} recorded since timing was enabled."""
        ms = np.zeros(len(STAGES))
        n = np.zeros(len(STAGES), dtype=np.int64)
        _check(load().purify_gb300_stage_times(self._h, _np_ptr(ms), _np_ptr(n)))
        return {s: (float(ms[k]), int(n[k])) for k, s in enumerate(STAGES)}

    # -- device path -------------------------------------------------------
    def _stream(self, stream):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        return ctypes.c_void_p(stream.cuda_stream)

    def forward_into(self, x, y, stream=None):
        _check(load().purify_gb300_forward(self._h, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(y.data_ptr()), self._stream(stream)))
        return y

    def adjoint_into(self, y, x, stream=None):
        _check(load().purify_gb300_adjoint(self._h, ctypes.c_void_p(y.data_ptr()),
                                           ctypes.c_void_p(x.data_ptr()), self._stream(stream)))
        return x

    def normal(self, x, stream=None):
        """Phi^H Phi x for a CUDA tensor x (imsizey*imsizex values), the
        combined degrid/grid operator (init_grid_degrid_operator_2d)."""
        import torch
        self._check_device_tensor(x, self.imsizey * self.imsizex)
        out = torch.empty_like(x)
        return self.normal_into(x, out, stream)

    def normal_into(self, x, out, stream=None):
        _check(load().purify_gb300_normal(self._h, ctypes.c_void_p(x.data_ptr()),
                                          ctypes.c_void_p(out.data_ptr()), self._stream(stream)))
        return out

    def forward_backward(self, y, x0=None, stream=None, **params):
        """Forward-backward iterations of min 1/2 ||y - Phi x||^2 + gamma ||x||_1
        on the device (purify_gb300_forward_backward).  y: CUDA tensor of M
        values; x0: start (zeros when None).  Keyword parameters: iterations,
        step, gamma_scale, update_scale, update_tol, update_iters,
        real_constraint, positive_constraint.  Returns (x, gammas)."""
        import torch
        self._check_device_tensor(y, self.M)
        n = self.imsizey * self.imsizex
        x = torch.zeros(n, dtype=self.complex_dtype, device=y.device) if x0 is None else x0.clone()
        p = FbParams()
        load().purify_gb300_fb_default_params(ctypes.byref(p))
        for k, v in params.items():
            if not hasattr(p, k):
                raise PurifyError(1, "unknown forward-backward parameter %s" % k)
            setattr(p, k, type(getattr(p, k))(v))
        gammas = np.zeros(max(int(p.iterations), 1))
        _check(load().purify_gb300_forward_backward(self._h, ctypes.c_void_p(y.data_ptr()),
                                                    ctypes.c_void_p(x.data_ptr()), ctypes.byref(p),
                                                    _np_ptr(gammas), self._stream(stream)))
        return x, gammas[:int(p.iterations)]

    def degrid_into(self, grid, vis, stream=None):
        """G alone: grid (ftsizev*ftsizeu) -> vis (M), device tensors."""
        _check(load().purify_gb300_degrid(self._h, ctypes.c_void_p(grid.data_ptr()),
                                          ctypes.c_void_p(vis.data_ptr()), self._stream(stream)))
        return vis

    def grid_into(self, vis, grid, stream=None):
        """G^H alone: vis (M) -> grid (ftsizev*ftsizeu), device tensors."""
        _check(load().purify_gb300_grid(self._h, ctypes.c_void_p(vis.data_ptr()),
                                        ctypes.c_void_p(grid.data_ptr()), self._stream(stream)))
        return grid

    def grid_no_alloc_into(self, vis, grid, stream=None):
        """G^H alone with no device allocation: the scratch is the library's
        fixed array (purify_gb300_grid_no_alloc).  Same result as grid_into."""
        _check(load().purify_gb300_grid_no_alloc(self._h, ctypes.c_void_p(vis.data_ptr()),
                                                 ctypes.c_void_p(grid.data_ptr()),
                                                 self._stream(stream)))
        return grid

    def grid_no_alloc_bytes(self):
        """Scratch bytes the allocation-free G^H needs for this operator."""
        n = ctypes.c_int64()
        _check(load().purify_gb300_grid_no_alloc_bytes(self._h, ctypes.byref(n)))
        return n.value

    def _check_device_tensor(self, t, n):
        if not t.is_cuda or t.dtype != self.complex_dtype or not t.is_contiguous() or t.numel() != n:
            raise PurifyError(1, "expected a contiguous CUDA %s tensor of %d values"
                              % (self.complex_dtype, n))

    # -- reference-facing apply -------------------------------------------
    def forward(self, x, stream=None):
        """Phi x.  x: imsizey*imsizex values."""
        n = self.imsizey * self.imsizex
        if _is_torch(x):
            import torch
            self._check_device_tensor(x, n)
            y = torch.empty(self.M, dtype=self.complex_dtype, device=x.device)
            return self.forward_into(x, y, stream)
        x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
        if x.size != n:
            raise PurifyError(1, "image vector has %d values, expected %d" % (x.size, n))
        y = np.empty(self.M, dtype=np.complex128)
        _check(load().purify_gb300_forward_host(self._h, _np_ptr(x), _np_ptr(y)))
        return y

    def adjoint(self, y, stream=None):
        """Phi^H y.  y: M values."""
        n = self.imsizey * self.imsizex
        if _is_torch(y):
            import torch
            self._check_device_tensor(y, self.M)
            x = torch.empty(n, dtype=self.complex_dtype, device=y.device)
            return self.adjoint_into(y, x, stream)
        y = np.ascontiguousarray(y, dtype=np.complex128).ravel()
        if y.size != self.M:
            raise PurifyError(1, "visibility vector has %d values, expected %d" % (y.size, self.M))
        x = np.empty(n, dtype=np.complex128)
        _check(load().purify_gb300_adjoint_host(self._h, _np_ptr(y), _np_ptr(x)))
        return x


def init_degrid_operator_2d(u, v, w, weights, imsizey, imsizex, oversample_ratio=2.0,
                            power_iters=100, power_tol=1e-4, kernel="kb", Ju=4, Jv=4,
                            w_term=False, Jw=6, cellx=1.0, celly=1.0, precision="fp32",
                            device=0):
    """The reference's factory signature (operators.h:373-380), u/v in pixels."""
    return MeasurementOperator(u, v, w, weights, imsizey, imsizex, oversample_ratio, power_iters,
                               power_tol, kernel, Ju, Jv, w_term, Jw, cellx, celly, precision,
                               device)


class Batch:
    """Many channels (each its own coverage and image size; one kernel, J and
    oversampling) applied together: grouped launches recorded once into a
    CUDA graph and replayed.  The reference applies such a set operator by
    operator (init_combine_operators, cpp/purify/operators.h:513-527).

    ``channels`` is a list of dicts with keys u, v (grid pixels), imsizey,
    imsizex and optionally weights.  ``tuning`` None runs the autotuner; a dict
    with tile / max_per_item / degrid_threads / grid_threads fixes it."""

    def __init__(self, channels, oversample_ratio=2.0, kernel="kb", J=4, precision="fp32",
                 device=0, tuning=None):
        L = load()
        n = len(channels)
        arr = (Channel * max(n, 1))()
        self._keep = []
        self.M, self.imsizes = [], []
        for k, ch in enumerate(channels):
            u = np.ascontiguousarray(ch["u"], dtype=np.float64).ravel()
            v = np.ascontiguousarray(ch["v"], dtype=np.float64).ravel()
            if u.size != v.size:
                raise PurifyError(1, "channel %d: u and v differ in length" % k)
            wt = ch.get("weights")
            wt = None if wt is None else np.ascontiguousarray(wt, dtype=np.complex128).ravel()
            self._keep += [u, v, wt]
            arr[k] = Channel(_np_ptr(u), _np_ptr(v), _np_ptr(wt), u.size, int(ch["imsizey"]),
                             int(ch["imsizex"]))
            self.M.append(int(u.size))
            self.imsizes.append((int(ch["imsizey"]), int(ch["imsizex"])))
        h = ctypes.c_void_p()
        t = None
        if tuning:
            t = BatchTuning(int(tuning.get("tile", 0)), int(tuning.get("max_per_item", 0)),
                            int(tuning.get("degrid_threads", 0)),
                            int(tuning.get("grid_threads", 0)), int(tuning.get("cell_group", 0)),
                            int(tuning.get("fft_columns", 0)))
        _check(L.purify_gb300_batch_create(arr, n, float(oversample_ratio),
                                           KERNELS[kernel] if isinstance(kernel, str) else int(kernel),
                                           int(J), PRECISIONS[precision], int(device),
                                           ctypes.byref(t) if t is not None else None,
                                           ctypes.byref(h)))
        self._keep = None
        self._h = h
        self.nch = n
        self.precision = precision
        self.device = int(device)
        self._bound = None

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().purify_gb300_batch_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def complex_dtype(self):
        import torch
        return torch.complex64 if self.precision == "fp32" else torch.complex128

    @property
    def tuning(self):
        t = BatchTuning()
        _check(load().purify_gb300_batch_get_tuning(self._h, ctypes.byref(t)))
        return {"tile": t.tile, "max_per_item": t.max_per_item,
                "degrid_threads": t.degrid_threads, "grid_threads": t.grid_threads,
                "cell_group": t.cell_group, "fft_columns": t.fft_columns}

    def info(self):
        i = BatchInfo()
        _check(load().purify_gb300_batch_info_get(self._h, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in BatchInfo._fields_}

    def _stream(self, stream):
        import torch
        if stream is None:
            stream = torch.cuda.current_stream(self.device)
        return ctypes.c_void_p(stream.cuda_stream)

    def _ptrs(self, tensors, sizes, what):
        if tensors is None:
            return None
        if len(tensors) != self.nch:
            raise PurifyError(1, "%s: expected %d tensors" % (what, self.nch))
        out = (ctypes.c_void_p * self.nch)()
        for k, (t, n) in enumerate(zip(tensors, sizes)):
            if (not t.is_cuda or t.dtype != self.complex_dtype or not t.is_contiguous()
                    or t.numel() != n):
                raise PurifyError(1, "%s[%d]: expected a contiguous CUDA %s tensor of %d values"
                                  % (what, k, self.complex_dtype, n))
            out[k] = t.data_ptr()
        return out

    def bind(self, x_in=None, vis=None, x_out=None, stream=None):
        """Binds per-channel device tensors (lists of nch tensors)."""
        npix = [a * b for a, b in self.imsizes]
        xi = self._ptrs(x_in, npix, "x_in")
        vi = self._ptrs(vis, self.M, "vis")
        xo = self._ptrs(x_out, npix, "x_out")
        _check(load().purify_gb300_batch_bind(self._h, xi, vi, xo, self._stream(stream)))
        self._bound = (x_in, vis, x_out)  # keep the tensors alive while bound

    def apply(self, directions=3, stream=None):
        """1: vis = Phi x_in; 2: x_out = Phi^H vis; 3: both in turn."""
        _check(load().purify_gb300_batch_apply(self._h, int(directions), self._stream(stream)))

    def time(self, what=3, reps=10):
        """Average device ms of one replay (1, 2, 3 as apply; 8 / 16 the
        grouped degrid / grid launch alone) on the batch's own buffers."""
        ms = ctypes.c_double()
        _check(load().purify_gb300_batch_time(self._h, int(what), int(reps), ctypes.byref(ms)))
        return ms.value

    def power_method(self, iters=100, tol=1e-4):
        n = np.zeros(self.nch)
        _check(load().purify_gb300_batch_power_method(self._h, int(iters), float(tol), _np_ptr(n)))
        return n

    def set_norms(self, norms):
        n = np.ascontiguousarray(norms, dtype=np.float64)
        if n.size != self.nch:
            raise PurifyError(1, "expected %d norms" % self.nch)
        _check(load().purify_gb300_batch_set_norms(self._h, _np_ptr(n)))

    @property
    def norms(self):
        n = np.zeros(self.nch)
        _check(load().purify_gb300_batch_get_norms(self._h, _np_ptr(n)))
        return n


class Server:
    """Request server on one GPU: coverages resident on the device, requests
    admitted by an HBM budget and run concurrently on `slots` streams, each
    with its own workspace (see include/purify_gb300.h).  Host vectors are
    complex128 numpy arrays."""

    def __init__(self, device=0, slots=8, hbm_budget=8 << 30, norm_slots=0):
        L = load()
        cfg = ServerConfig(int(device), int(slots), int(hbm_budget), int(norm_slots))
        h = ctypes.c_void_p()
        _check(L.purify_gb300_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._cov = []       # (M, N) per coverage
        self._out = {}       # ticket -> output arrays

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().purify_gb300_server_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_coverage(self, u, v, w=None, weights=None, imsizey=256, imsizex=256,
                     oversample_ratio=2.0, power_iters=0, power_tol=1e-4, kernel="kb", Ju=4,
                     Jv=4, w_term=False, Jw=6, cellx=1.0, celly=1.0, precision="fp32",
                     jw_rows=None):
        a, keep = _create_args(u, v, w, weights, imsizey, imsizex, oversample_ratio, power_iters,
                               power_tol, kernel, Ju, Jv, w_term, Jw, cellx, celly, precision, 0,
                               jw_rows)
        cid = ctypes.c_int32()
        _check(load().purify_gb300_server_add_coverage(self._h, ctypes.byref(a), ctypes.byref(cid)))
        del keep
        self._cov.append((int(a.M), int(imsizey) * int(imsizex)))
        return cid.value

    def _request(self, coverage, kind, x=None, vis=None, iters=50, tol=1e-4):
        if not 0 <= int(coverage) < len(self._cov):
            raise PurifyError(1, "unknown coverage %d" % coverage)
        M, N = self._cov[coverage]
        k = REQUEST_KINDS[kind] if isinstance(kind, str) else int(kind)
        rq = Request()
        rq.coverage, rq.kind, rq.iters, rq.tol = int(coverage), k, int(iters), float(tol)
        keep, outs = [], {}
        if k in (1, 3):
            x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
            if x.size != N:
                raise PurifyError(1, "image vector has %d values, expected %d" % (x.size, N))
            keep.append(x)
            rq.x_in = _np_ptr(x)
            outs["vis"] = np.empty(M, dtype=np.complex128)
            rq.vis_out = _np_ptr(outs["vis"])
        if k == 2:
            vis = np.ascontiguousarray(vis, dtype=np.complex128).ravel()
            if vis.size != M:
                raise PurifyError(1, "visibility vector has %d values, expected %d" % (vis.size, M))
            keep.append(vis)
            rq.vis_in = _np_ptr(vis)
        if k in (2, 3):
            outs["x"] = np.empty(N, dtype=np.complex128)
            rq.x_out = _np_ptr(outs["x"])
        return rq, keep, outs

    def request_bytes(self, coverage, kind, iters=50):
        if not 0 <= int(coverage) < len(self._cov):
            raise PurifyError(1, "unknown coverage %d" % coverage)
        M, N = self._cov[coverage]
        rq, _, _ = self._request(coverage, kind, np.zeros(N, np.complex128),
                                 np.zeros(M, np.complex128), iters)
        b = ctypes.c_int64()
        _check(load().purify_gb300_server_request_bytes(self._h, ctypes.byref(rq), ctypes.byref(b)))
        return b.value

    def submit(self, coverage, kind, x=None, vis=None, iters=50, tol=1e-4):
        """Queues a request ("forward", "adjoint", "forward_adjoint", "norm");
        returns its ticket.  Inputs are copied before this returns."""
        rq, keep, outs = self._request(coverage, kind, x, vis, iters, tol)
        t = ctypes.c_int64()
        _check(load().purify_gb300_server_submit(self._h, ctypes.byref(rq), ctypes.byref(t)))
        del keep
        self._out[t.value] = outs
        return t.value

    def wait(self, ticket, timeout=None):
        """The request's result dict (status, norm, iterations, queue_ms,
        run_ms, latency_ms, device_bytes, vis / x outputs), or None if it is
        still running after `timeout` seconds."""
        r = Result()
        rc = load().purify_gb300_server_wait(self._h, int(ticket),
                                             -1.0 if timeout is None else float(timeout),
                                             ctypes.byref(r))
        if rc == 7:
            return None
        _check(rc)
        out = {f: getattr(r, f) for f, _ in Result._fields_}
        out.update(self._out.pop(ticket, {}))
        return out

    def stats(self):
        st = ServerStats()
        _check(load().purify_gb300_server_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}



class PsfConvolve:
    """Convolution with the operator's point-spread function, the
    image-domain approximation of Phi^H Phi (init_psf_convolve_2d,
    cpp/purify/compact_operators.h:279-307), on CUDA tensors."""

    def __init__(self, op, power_iters=100, power_tol=1e-4):
        h = ctypes.c_void_p()
        _check(load().purify_gb300_psf_create(op.handle, int(power_iters), float(power_tol),
                                              ctypes.byref(h)))
        self._h = h
        self.op = op

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().purify_gb300_psf_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def norm(self):
        n = ctypes.c_double()
        _check(load().purify_gb300_psf_norm(self._h, ctypes.byref(n)))
        return n.value

    def __call__(self, x, out=None, stream=None):
        import torch
        self.op._check_device_tensor(x, self.op.imsizey * self.op.imsizex)
        out = torch.empty_like(x) if out is None else out
        _check(load().purify_gb300_psf_apply(self._h, ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()),
                                             self.op._stream(stream)))
        return out
