#!/usr/bin/env python
"""Benchmark of the GB300 measurement operator (degrid + grid Mvis/s).

A step is one forward Phi x followed by one adjoint Phi^H y (y = the forward
result) on the 1024^2-image workload: 2048^2 grid (oversampling 2),
10^7 visibilities (70% Gaussian core with sigma = 0.15 N, 30% uniform),
Kaiser-Bessel J = 6, complex<float> arithmetic.  ``value`` is visibilities
per second through degrid + grid with inputs resident in HBM; ``e2e`` is the
same metric through the host complex<double> entry points, host<->device
copies included.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the CPU FP64 restatement of the reference
operator (CSR G and G^H, row-parallel SpMV, unitary FFT) on the host cores.
Under torchrun (N > 1) every rank runs an independent replica (weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "purify-1_gb300"))

METRIC = "degrid+grid Mvis/s at 1024^2 (Phi then Phi^H per step), FP32 vs FP64 plain"
WORKLOAD = ("1024^2 image, 2048^2 grid, M=1e7 visibilities (70% Gaussian core sigma=0.15N, "
            "30% uniform), Kaiser-Bessel Ju=Jv=6, weights 1")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=["imaging", "wproj", "batch", "serve"],
                   default="imaging",
                   help="imaging: the 1024^2 / 1e7 headline; wproj: 2048^2 / 2e7 w-projection; "
                        "batch: 64 channels in one graph-replayed grouped step; serve: Poisson "
                        "request stream on 16 resident coverages")
    p.add_argument("--rate", type=float, default=100.0, help="serve: requests per second")
    p.add_argument("--requests", type=int, default=400, help="serve: timed requests")
    p.add_argument("--slots", type=int, default=8, help="serve: requests in flight at most")
    p.add_argument("--budget-gb", type=float, default=24.0, help="serve: HBM budget of requests")
    p.add_argument("--channels", type=int, default=64, help="channels of the batch workload")
    p.add_argument("--M", type=int, default=0, help="visibilities (0: the workload's own)")
    p.add_argument("--imsize", type=int, default=1024)
    p.add_argument("--J", type=int, default=6)
    p.add_argument("--cpu-sample", type=int, default=1_000_000,
                   help="visibilities of the extrapolated CPU sample kept beside the full-size "
                        "CPU figure (0: none)")
    p.add_argument("--cpu-pairs", type=int, default=10,
                   help="timed Phi / Phi^H pairs of the full-size CPU baseline")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=20, help="0 skips the end-to-end leg")
    p.add_argument("--power-iters", type=int, default=20,
                   help="power-method rounds for the norm before timing (0: norm 1)")
    p.add_argument("--threads", type=int, default=0, help="CTA threads (tuning)")
    p.add_argument("--max-per-item", type=int, default=0)
    p.add_argument("--tile", type=int, default=0, help="uv tile edge (tuning)")
    p.add_argument("--cell-group", type=int, default=0,
                   help="base cells per work item along each axis: 1, 2, or 0 for the default")
    p.add_argument("--class-cap", type=int, default=0,
                   help="most items of one bank class per batch (0: default; tuning)")
    p.add_argument("--grid-walk", type=int, default=0,
                   help="1: G^H of Phi^H by the column walk instead of work items (tuning)")
    p.add_argument("--fft-columns", type=int, default=0,
                   help="1: cuFFT's column plan instead of the column pass (tuning)")
    p.add_argument("--normal-pass", type=int, default=0,
                   help="1: the normal operator's G^H G in one pass over each task (tuning)")
    p.add_argument("--keep-store", type=int, default=0,
                   help="1: Phi stores its caller-ordered output at L2 evict-last priority (tuning)")
    p.add_argument("--fused-permute", type=int, default=-1,
                   help="1: degrid/grid touch caller order directly, 0: gather kernels, "
                        "-1: default per direction (tuning)")
    return p.parse_args()


def tuning_of(args):
    """Tuning dict of the --threads / --max-per-item / --tile flags (None: defaults)."""
    t = {k: v for k, v in (("threads", args.threads), ("max_per_item", args.max_per_item),
                           ("tile", args.tile), ("cell_group", args.cell_group),
                           ("class_cap", args.class_cap), ("keep_store", args.keep_store),
                           ("fft_columns", args.fft_columns), ("grid_walk", args.grid_walk),
                           ("normal_pass", args.normal_pass))
         if v}
    if args.fused_permute >= 0:
        t["fused_permute"] = args.fused_permute
    return t or None


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(args, seed):
    from purify_gb300 import synthetic
    n = args.imsize
    if not args.M:
        args.M = 10_000_000
    u, v = synthetic.mixed_uv(args.M, 2 * n, 2 * n, 0.7, 0.15, seed=seed)
    x = synthetic.sky_image(n, n, seed=seed)
    return u, v, x


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of each kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append((time.time(), parts))

    def window(self, t0, t1):
        return [p for (t, p) in self.rows if t0 <= t <= t1]

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, rows):
        if not rows:
            return None

        def num(s):
            try:
                return float(s)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# --------------------------------------------------------------- CPU oracle --
def cpu_reference(u, v, x, imsize, J, pairs=10, warmup=1, sample=1_000_000):
    """Times the FP64 oracle (the reference algorithm restated: explicit CSR G
    and G^H, row-parallel OpenMP SpMV, unitary FFT) on the full workload:
    construction once, then `warmup` untimed and `pairs` timed Phi / Phi^H
    pairs; the value is M over the median pair.  A `sample`-visibility
    subsample with a per-visibility extrapolation is kept beside it for
    comparison with earlier figures (0 skips it)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    threads = oracle.get_threads()
    M = u.size
    t0 = time.perf_counter()
    op = oracle.Operator(u, v, None, None, imsize, imsize, 2.0, kernel="kb", Ju=J, Jv=J)
    t_create = time.perf_counter() - t0
    tf, ta, tp = [], [], []
    for k in range(warmup + pairs):
        t0 = time.perf_counter()
        y = op.forward(x)
        t1 = time.perf_counter()
        op.adjoint(y)
        t2 = time.perf_counter()
        if k >= warmup:
            tf.append(t1 - t0)
            ta.append(t2 - t1)
            tp.append(t2 - t0)
    nnz = op.nnz
    del op
    t_pair = statistics.median(tp)
    out = {
        "value": M / t_pair / 1e6, "unit": "Mvis/s", "cores": threads, "kind": "port",
        "sample": ("the full workload (M=%d, %d^2 grid, %d non-zeros in G and again in G^H): "
                   "Phi then Phi^H of the FP64 oracle (CSR G/G^H, OpenMP SpMV, radix-2 FFT), "
                   "median of %d timed pairs after %d untimed; construction %.1f s not timed"
                   % (M, 2 * imsize, nnz, pairs, warmup, t_create)),
        "ms_per_pair": t_pair * 1e3, "ms_forward": statistics.median(tf) * 1e3,
        "ms_adjoint": statistics.median(ta) * 1e3, "create_s": t_create,
        "host_bytes_G_and_GH": 2 * nnz * 20, "timed": True,
    }
    if sample and sample < M:
        idx = np.random.default_rng(123).choice(M, sample, replace=False)
        op0 = oracle.Operator(u[:0], v[:0], None, None, imsize, imsize, 2.0, kernel="kb", Ju=J,
                              Jv=J)
        ops = oracle.Operator(u[idx], v[idx], None, None, imsize, imsize, 2.0, kernel="kb",
                              Ju=J, Jv=J)

        def pair_time(o):
            ts = []
            for k in range(3):
                t0 = time.perf_counter()
                o.adjoint(o.forward(x))
                if k >= 1:
                    ts.append(time.perf_counter() - t0)
            return statistics.median(ts)
        t_fixed, t_s = pair_time(op0), pair_time(ops)
        t_ext = t_fixed + max(t_s - t_fixed, 0.0) / sample * M
        out["sample_extrapolated"] = {
            "value": M / t_ext / 1e6, "visibilities": sample,
            "how": "per-visibility cost of a %d-visibility sample extrapolated to M" % sample}
    return out


def host_memory_gb():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemTotal:"):
                    return int(line.split()[1]) / 2**20
    except Exception:
        pass
    return None


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    u, v, x = workload(args, seed=0)
    # each step: one Phi / Phi^H pair of the full workload
    cb = cpu_reference(u, v, x, args.imsize, args.J, pairs=max(1, args.steps),
                       warmup=max(1, args.warmup), sample=0)
    line = {
        "metric": METRIC, "value": cb["value"], "unit": "Mvis/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_pair"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded (PCG64) coverage and point-source + Gaussian-blob sky",
        "config": {"workload": WORKLOAD, "global_visibilities": args.M,
                   "parallelism": "host threads", "host_memory_gb": host_memory_gb()},
        "impl": "reference", "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------- GPU ----
def kernel_bytes(info, s, caller_order_out=True, caller_order_in=True):
    """Bytes each gridding-chain kernel's own arguments carry per launch
    (complex values of s bytes): what the kernel must read or write at least
    once, independent of how it does it.  Weights are not among them: a
    weighted operator applies them in separate elementwise passes.

    degrid: the grid once, per slot t (s) [+ caller index (4) when it writes
            caller order], lane codes and batch headers, and the M
            visibilities it writes;
    grid:   per slot t (s), lane codes and headers, the task windows it
            writes, and either the slot-ordered visibility (s per slot) or,
            when it gathers caller order itself, the caller index (4 per
            slot) and the M caller-ordered visibilities;
    expand: per slot the caller index (4) and the slot written (s), and the M
            caller-ordered visibilities read (only when grid reads slots);
    fold:   the task windows read and the grid written."""
    S, M = info["slots"], info["M"]
    NuNv = info["ftsizeu"] * info["ftsizev"]
    items = info["work_items"]
    lanes = 4 * items + 8 * (items // 32)
    windows = s * info["tasks"] * info["window_cells"]
    out = {
        "degrid": s * NuNv + s * S + (4 * S if caller_order_out else 0) + lanes + s * M,
        "grid": (s * S + 4 * S + s * M if caller_order_in else 2 * s * S) + lanes + windows,
        "fold": windows + s * NuNv,
    }
    if not caller_order_in:
        out["expand"] = 4 * S + s * S + s * M
    nw = info.get("walk_tasks", 0)
    if nw:
        # the column walk of Phi^H: per slot (S = M) t and the visibility,
        # per task 32 x 32 counts and 33 column starts, and its window
        wwin = s * nw * info["window_cells"]
        out["grid"] = 2 * s * M + 4 * (32 * 32 + 33) * nw + wwin
        out["expand"] = 4 * M + 2 * s * M
        out["fold"] = wwin + s * NuNv
    return out


def roofline_entry(kern, alg, dur_s, peak, peak_kind, traffic, formula_bytes=None):
    """achieved / frac on the kernel's own bytes, frac_dram on its profiled
    DRAM traffic, and (when given) the per-visibility formula's bytes
    M (16 + 2 s) + s NuNv (u, v, weight and visibility per visibility, the
    grid once) beside them."""
    achieved = alg / dur_s / 1e9
    r = {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
         "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes": alg,
         "duration_ms": dur_s * 1e3, "traffic": traffic,
         "frac_dram": (traffic / dur_s / 1e9 / peak) if traffic else None}
    if formula_bytes:
        r["formula_bytes"] = formula_bytes
        r["frac_formula_bytes"] = formula_bytes / dur_s / 1e9 / peak
    return r



def run_gb300(args):
    import torch
    import purify_gb300 as pgb

    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pgb.build()

    u, v, x = workload(args, seed=rank)
    n, M, N = args.imsize, args.M, args.imsize * args.imsize
    kw = dict(imsizey=n, imsizex=n, oversample_ratio=2.0, kernel="kb", Ju=args.J, Jv=args.J,
              device=local)
    t0 = time.perf_counter()
    op = pgb.MeasurementOperator(u, v, None, None, power_iters=0, precision="fp32",
                                 tuning=tuning_of(args), **kw)
    t_create = time.perf_counter() - t0
    t0 = time.perf_counter()
    norm = op.power_method(args.power_iters, 1e-4) if args.power_iters > 0 else 1.0
    t_power = time.perf_counter() - t0
    info = op.info()

    stream = torch.cuda.current_stream(dev)
    xd = torch.from_numpy(x).to(torch.complex64).to(dev)
    yd = torch.empty(M, dtype=torch.complex64, device=dev)
    xo = torch.empty(N, dtype=torch.complex64, device=dev)

    def step():
        op.forward_into(xd, yd, stream)
        op.adjoint_into(yd, xo, stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        time.sleep(0.5)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    w0 = time.time()
    evs[0].record(stream)
    for k in range(args.steps):
        step()
        evs[k + 1].record(stream)
    torch.cuda.synchronize(dev)
    w1 = time.time()
    if dist:
        dist.barrier()
    total_ms = evs[0].elapsed_time(evs[-1])
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    # forward and adjoint alone, and the normal operator Phi^H Phi (slot
    # order between its halves, no permutations), each over the same number
    # of steps (after the timed steps, so the headline number is unaffected)
    directions = {}
    for name, fn in (("forward", lambda: op.forward_into(xd, yd, stream)),
                     ("adjoint", lambda: op.adjoint_into(yd, xo, stream)),
                     ("normal", lambda: op.normal_into(xd, xo, stream))):
        fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
        directions[name] = {"ms": ms, "mvis_s": M / (ms * 1e-3) / 1e6}
    # adjoint dot-product test at full size, |<Phi x, y> - <x, Phi^H y>| /
    # (||Phi x|| ||y||), with a seeded random y; FP64 sums on the device
    gen = torch.Generator(device=dev).manual_seed(11)
    yr = torch.complex(torch.randn(M, device=dev, generator=gen),
                       torch.randn(M, device=dev, generator=gen)).to(torch.complex64)
    xa = torch.empty(N, dtype=torch.complex64, device=dev)
    op.forward_into(xd, yd, stream)
    op.adjoint_into(yr, xa, stream)
    torch.cuda.synchronize(dev)
    lhs = torch.vdot(yr.to(torch.complex128), yd.to(torch.complex128))
    rhs = torch.vdot(xa.to(torch.complex128), xd.to(torch.complex128))
    adjoint_test = float(abs(lhs - rhs) / (torch.linalg.vector_norm(yd.to(torch.complex128)) *
                                         torch.linalg.vector_norm(yr.to(torch.complex128))))
    del yr, xa
    # per-stage breakdown in a separate pass (the events between stages are
    # not in the timed steps)
    op.stage_timing(True)
    for _ in range(max(3, min(args.steps, 20))):
        step()
    stages = op.stage_times()
    op.stage_timing(False)
    clocks = None
    if sampler:
        time.sleep(0.3)
        sampler.stop()
        clocks = sampler.summary(sampler.window(w0 - 0.25, w1 + 0.25)) or sampler.summary(
            sampler.rows)
    ms_per_step = total_ms / args.steps
    if dist:
        t = torch.tensor([ms_per_step], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_per_step = float(t.item())
    value = world * M / (ms_per_step * 1e-3) / 1e6
    # Phi^H's grid kernel gathers the caller-ordered visibilities itself
    # unless the tuning asks for the slot-ordered path or the column walk
    gather_in_grid = (args.fused_permute == 1 or (args.fused_permute < 0 and args.J >= 4)) \
        and not args.grid_walk

    out = {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded (PCG64) coverage and point-source + Gaussian-blob sky",
        "config": {"workload": WORKLOAD, "global_visibilities": world * M,
                   "l2": "inputs larger than L2 (about 300 MB of coverage state and "
                         "visibilities read per step vs 129 MB L2); the 80 MB caller-ordered "
                         "visibility vector, Phi's output and Phi^H's input, is read by the "
                         "adjoint's gather at L2 evict-last priority and so stays in L2 for "
                         "the next step's degrid, as in a solver's Phi / Phi^H loop",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "latency_ms": {"p50": float(np.percentile(per_step, 50)),
                       "p99": float(np.percentile(per_step, 99))},
        "create_s": t_create, "power_method_s": t_power, "norm": norm,
        "stages_ms_per_launch": {k: (ms / nl if nl else None) for k, (ms, nl) in stages.items()},
        "directions": directions,
        "adjoint_dot_test_fp32": adjoint_test,
        # own kernels per step: the forward row and column passes, degrid
        # (compact after it on the slot-ordered forward, --fused-permute 0),
        # grid (gathering caller order itself; expand before it when it does
        # not), fold, the inverse column and row passes (cuFFT's column plan
        # instead of the column passes with --fft-columns 1)
        "gpu_launches": ((5 if args.fft_columns == 1 else 7) + (0 if gather_in_grid else 1) +
                         (1 if args.fused_permute == 0 else 0)) * args.steps,
        "clocks": clocks,
    }

    # roofline of the dominant kernel (degrid or grid): the bytes its own
    # arguments carry (kernel_bytes), the per-visibility formula beside it,
    # and the profiled DRAM traffic per launch
    s = 8
    kb = kernel_bytes(info, s, caller_order_out=True, caller_order_in=gather_in_grid)
    kern = max(("degrid", "grid"), key=lambda k: stages[k][0] / max(stages[k][1], 1))
    dur = stages[kern][0] / max(stages[kern][1], 1) * 1e-3
    peak, peak_kind = measured_peak()
    # the profiled traffic belongs to the headline workload only
    headline = (M == 10_000_000 and n == 1024 and args.J == 6 and not tuning_of(args))
    traffic = profiled_traffic().get(
        "grid_caller_order" if kern == "grid" and gather_in_grid else kern) if headline else None
    out["roofline"] = roofline_entry(kern, kb[kern], dur, peak, peak_kind, traffic,
                                     M * (16 + 2 * s) + s * info["ftsizeu"] * info["ftsizev"])
    out["kernel_bytes"] = kb
    # whole-step HBM view: B_fwd + B_adj of the per-visibility formula (c64)
    NuNv = info["ftsizeu"] * info["ftsizev"]
    b_step = 2 * M * (16 + 2 * s) + s * (7 * NuNv + 3 * N)
    out["step_roofline"] = {"algorithmic_bytes": b_step,
                            "achieved_gbs": b_step / (ms_per_step * 1e-3) / 1e9,
                            "frac": b_step / (ms_per_step * 1e-3) / 1e9 / peak}

    # FP32 vs FP64 GPU, same coverage and norm
    if not args.no_fp64:
        op64 = pgb.MeasurementOperator(u, v, None, None, power_iters=0, precision="fp64",
                                       tuning=tuning_of(args), **kw)
        op64.set_norm(norm)
        x64 = torch.from_numpy(x).to(dev)
        y64 = torch.empty(M, dtype=torch.complex128, device=dev)
        xo64 = torch.empty(N, dtype=torch.complex128, device=dev)
        for _ in range(max(1, args.warmup)):
            op64.forward_into(x64, y64, stream)
            op64.adjoint_into(y64, xo64, stream)
        k64 = max(3, args.steps // 5)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        for _ in range(k64):
            op64.forward_into(x64, y64, stream)
            op64.adjoint_into(y64, xo64, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms64 = e0.elapsed_time(e1) / k64
        # errors of the FP32 path against the FP64 path (same input)
        op.forward_into(xd, yd, stream)
        op64.forward_into(x64, y64, stream)
        op.adjoint_into(y64.to(torch.complex64), xo, stream)
        op64.adjoint_into(y64, xo64, stream)
        torch.cuda.synchronize(dev)
        f32y, f64y = yd.cpu().numpy(), y64.cpu().numpy()
        f32x, f64x = xo.cpu().numpy(), xo64.cpu().numpy()
        out["fp64"] = {"value": world * M / (ms64 * 1e-3) / 1e6, "ms_per_step": ms64,
                       "speedup_fp32_over_fp64": ms64 / ms_per_step}
        out["rel_l2_fp32_vs_fp64"] = {"forward": rel_l2(f32y, f64y), "adjoint": rel_l2(f32x, f64x)}
        # FP64 GPU vs the CPU FP64 oracle on a row sample (forward rows are independent)
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            idx = np.random.default_rng(7).choice(M, 20000, replace=False)
            ref = oracle.Operator(u[idx], v[idx], None, None, n, n, 2.0, kernel="kb", Ju=args.J,
                                  Jv=args.J)
            ref.set_norm(norm)
            yr = ref.forward(x)
            out["rel_l2_vs_oracle_forward_rows"] = {"fp32": rel_l2(f32y[idx], yr),
                                                    "fp64": rel_l2(f64y[idx], yr),
                                                    "rows": 20000}
        except Exception as e:  # the oracle is a checker only
            out["rel_l2_vs_oracle_forward_rows"] = {"error": str(e)}
        # the full-size adjoint of a y that is zero outside the row sample
        # equals the sampled operator's adjoint (G^H is linear in y)
        try:
            rng = np.random.default_rng(8)
            ys = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
            yfull = torch.zeros(M, dtype=torch.complex128)
            yfull[torch.from_numpy(idx)] = torch.from_numpy(ys)
            y64.copy_(yfull.to(dev))
            op64.adjoint_into(y64, xo64, stream)
            op.adjoint_into(y64.to(torch.complex64), xo, stream)
            torch.cuda.synchronize(dev)
            xr = ref.adjoint(ys)
            out["rel_l2_vs_oracle_adjoint_sample"] = {"fp32": rel_l2(xo.cpu().numpy(), xr),
                                                      "fp64": rel_l2(xo64.cpu().numpy(), xr),
                                                      "rows": int(idx.size)}
        except Exception as e:
            out["rel_l2_vs_oracle_adjoint_sample"] = {"error": str(e)}
        del op64

    # end to end through the host complex<double> entry points, pinned buffers
    if args.e2e_steps <= 0:
        if rank == 0:
            print(json.dumps(out), flush=True)
        if dist:
            dist.destroy_process_group()
        return
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.empty(M, dtype=torch.complex128).pin_memory()
    xoh = torch.empty(N, dtype=torch.complex128).pin_memory()
    xhn, yhn, xohn = xh.numpy(), yh.numpy(), xoh.numpy()
    import ctypes
    L = pgb.load()

    def e2e_step():
        pgb._check(L.purify_gb300_forward_host(op.handle, xhn.ctypes.data_as(ctypes.c_void_p),
                                               yhn.ctypes.data_as(ctypes.c_void_p)))
        pgb._check(L.purify_gb300_adjoint_host(op.handle, yhn.ctypes.data_as(ctypes.c_void_p),
                                               xohn.ctypes.data_as(ctypes.c_void_p)))
    e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_ms = []
    for _ in range(args.e2e_steps):
        t1 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t1) * 1e3)
    t_e2e = (time.perf_counter() - t0) / args.e2e_steps
    if dist:
        t = torch.tensor([t_e2e], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_e2e = float(t.item())
    out["e2e"] = {"value": world * M / t_e2e / 1e6, "unit": "Mvis/s", "ms_per_step": t_e2e * 1e3,
                  "steps": args.e2e_steps, "p50_ms": float(np.percentile(e2e_ms, 50)),
                  "max_ms": float(max(e2e_ms)),
                  "h2d_bytes_per_step": 16 * (N + M), "d2h_bytes_per_step": 16 * (M + N),
                  "api": "purify_gb300_forward_host + purify_gb300_adjoint_host "
                         "(complex<double> host vectors)"}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_reference(u, v, x, n, args.J, pairs=args.cpu_pairs,
                                            sample=args.cpu_sample)
        out["cpu_baseline"]["host_memory_gb"] = host_memory_gb()
    out["info"] = {k: info[k] for k in ("occupied_cells", "work_items", "tasks", "device_bytes",
                                        "kernel_fit_error")}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


WPROJ_WORKLOAD = ("2048^2 image, 4096^2 grid, M=2e7 visibilities (70% Gaussian core, 30% uniform),"
                  " w ~ U(-w_max, w_max), KB J=4 convolved with the small-angle w-kernel, "
                  "per-row support 4..24 taps per axis affine in |w|")


def run_wproj(args):
    """w-projection workload: Phi then Phi^H per step, FP32, one GPU."""
    import torch
    import purify_gb300 as pgb
    from purify_gb300 import synthetic
    pgb.build()
    dev = torch.device("cuda", 0)
    M = args.M or 20_000_000
    imsize = args.imsize if args.imsize != 1024 else 2048
    t0 = time.perf_counter()
    c = synthetic.config_wproj(M=M, imsize=imsize, seed=0)
    t_gen = time.perf_counter() - t0
    kw = dict(imsizey=imsize, imsizex=imsize, oversample_ratio=2.0, kernel="kb", Ju=4, Jv=4,
              w_term=True, Jw=6, cellx=c["cellx"], celly=c["celly"], jw_rows=c["jw_rows"])
    t0 = time.perf_counter()
    op = pgb.MeasurementOperator(c["u"], c["v"], c["w"], None, power_iters=0, precision="fp32",
                                 tuning=tuning_of(args), **kw)
    t_create = time.perf_counter() - t0
    norm = op.power_method(args.power_iters, 1e-4) if args.power_iters > 0 else 1.0
    info = op.info()
    stream = torch.cuda.current_stream(dev)
    N = imsize * imsize
    xd = torch.from_numpy(c["x"]).to(torch.complex64).to(dev)
    yd = torch.empty(M, dtype=torch.complex64, device=dev)
    xo = torch.empty(N, dtype=torch.complex64, device=dev)

    def step():
        op.forward_into(xd, yd, stream)
        op.adjoint_into(yd, xo, stream)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(0)
    time.sleep(0.5)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    w0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    w1 = time.time()
    time.sleep(0.3)
    sampler.stop()
    clocks = sampler.summary(sampler.window(w0 - 0.25, w1 + 0.25)) or sampler.summary(sampler.rows)
    ms = e0.elapsed_time(e1) / args.steps
    op.stage_timing(True)
    for _ in range(max(2, min(args.steps, 5))):
        step()
    stages = op.stage_times()
    op.stage_timing(False)
    taps = info["nnz"]
    NuNv = info["ftsizeu"] * info["ftsizev"]
    s8 = 8
    # Bytes the row-factor kernels' own arguments carry per launch: the
    # stored factors (info factor_values complex values, 2 rank S per row,
    # not the S^2 taps of explicit rows), per row its code (4), factor offset
    # (8) and weight (s), the M slot-ordered visibilities, and the grid once
    # (degrid) or the task windows (grid).  The per-visibility formula with
    # explicit FP32 rows (taps * s) is kept beside it.
    rows = info["factor_values"] * s8 + M * (4 + 8 + s8) + M * s8
    wbytes = {"degrid": rows + s8 * NuNv,
              "grid": rows + s8 * info["tasks"] * info["window_cells"]}
    formula = M * (16 + 2 * s8) + taps * s8 + s8 * NuNv
    kern = max(("degrid", "grid"), key=lambda k: stages[k][0] / max(stages[k][1], 1))
    dur = stages[kern][0] / max(stages[kern][1], 1) * 1e-3
    peak, peak_kind = measured_peak()
    out = {
        "metric": "w-projection degrid+grid Mvis/s (Phi then Phi^H per step), FP32",
        "value": M / (ms * 1e-3) / 1e6, "unit": "Mvis/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded (PCG64)",
        "config": {"workload": WPROJ_WORKLOAD, "taps": taps, "mean_support_sq": taps / M},
        "gtaps_per_s": 2 * taps / (ms * 1e-3) / 1e9,
        "stages_ms_per_launch": {k: (ms_ / nl if nl else None) for k, (ms_, nl) in stages.items()},
        "create_s": t_create, "generate_s": t_gen, "norm": norm,
        "device_bytes": info["device_bytes"], "factor_values": info["factor_values"],
        "clocks": clocks, "kernel_bytes": wbytes,
        "roofline": roofline_entry(kern, wbytes[kern], dur, peak, peak_kind, None, formula),
        # own kernels per step: the forward row pass, w degrid, the compaction
        # into caller order, the gather into slot order, w grid, fold, the
        # inverse row pass (the 4096-row columns go through cuFFT)
        "gpu_launches": 7 * args.steps,
    }
    # FP32 rows against the FP64 oracle on a row sample (rows are independent)
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        idx = np.random.default_rng(7).choice(M, 4000, replace=False)
        # The operator sees w - mean(w) over all rows; one extra row makes the
        # sample's mean equal to that, so the oracle centres w the same way.
        ws = c["w"][idx]
        w_extra = (idx.size + 1) * c["w"].mean() - ws.sum()
        ref = oracle.Operator(np.append(c["u"][idx], 0.0), np.append(c["v"][idx], 0.0),
                              np.append(ws, w_extra), None, imsize, imsize, 2.0, kernel="kb",
                              Ju=4, Jv=4, w_term=True,
                              jw_rows=np.append(c["jw_rows"][idx], 1).astype(np.int32),
                              cellx=c["cellx"], celly=c["celly"])
        ref.set_norm(norm)
        op.forward_into(xd, yd, stream)
        torch.cuda.synchronize(dev)
        y = yd.cpu().numpy()[idx]
        yr = ref.forward(c["x"])[:-1]
        out["rel_l2_vs_oracle_forward_rows"] = {"fp32": rel_l2(y, yr), "rows": int(idx.size)}
        if not args.no_cpu_baseline:
            t0 = time.perf_counter()
            for _ in range(2):
                yy = ref.forward(c["x"])
                ref.adjoint(yy)
            t_s = (time.perf_counter() - t0) / 2
            op0 = oracle.Operator(c["u"][:0], c["v"][:0], c["w"][:0], None, imsize, imsize, 2.0,
                                  kernel="kb", Ju=4, Jv=4, w_term=True)
            t0 = time.perf_counter()
            yy = op0.forward(c["x"])
            op0.adjoint(yy)
            t_fix = time.perf_counter() - t0
            t_full = t_fix + max(t_s - t_fix, 0) * taps / max(ref.nnz, 1)
            out["cpu_baseline"] = {
                "value": M / t_full / 1e6, "unit": "Mvis/s", "cores": oracle.get_threads(),
                "kind": "port",
                "sample": "FP64 oracle on %d rows (%d taps); per-tap cost extrapolated to %d taps"
                          % (idx.size, ref.nnz, taps)}
    except Exception as e:
        out["rel_l2_vs_oracle_forward_rows"] = {"error": str(e)}
    print(json.dumps(out), flush=True)


BATCH_WORKLOAD = ("64 channels, image {256,512,1024}^2 drawn per channel, M log-uniform in "
                  "[1e4, 2e6], 70% Gaussian core sigma = 0.15 N (1 + 0.01 k) + 30% uniform, "
                  "KB J=4, FP32")


def run_batch(args):
    """Batched channels: one step = Phi then Phi^H of every channel, replayed
    from one CUDA graph; compared with the same applies made channel by
    channel through single operators."""
    import torch
    import purify_gb300 as pgb
    from purify_gb300 import synthetic
    pgb.build()
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    chans = synthetic.config_batch(args.channels, seed=0)
    t_gen = time.perf_counter() - t0
    Ms = [c["u"].size for c in chans]
    Mtot = int(sum(Ms))
    npix = [c["imsizey"] * c["imsizex"] for c in chans]
    t0 = time.perf_counter()
    b = pgb.Batch(chans, J=4, precision="fp32")
    t_create = time.perf_counter() - t0
    tuning = b.tuning
    if args.fft_columns:
        # the autotuned shapes with the other column transform (A/B)
        b.close()
        tuning["fft_columns"] = args.fft_columns
        b = pgb.Batch(chans, J=4, precision="fp32", tuning=tuning)
    t0 = time.perf_counter()
    norms = b.power_method(args.power_iters, 1e-4) if args.power_iters > 0 else np.ones(len(chans))
    t_power = time.perf_counter() - t0
    info = b.info()
    stream = torch.cuda.current_stream(dev)
    xs = [torch.from_numpy(c["x"]).to(torch.complex64).to(dev) for c in chans]
    vis = [torch.empty(m, dtype=torch.complex64, device=dev) for m in Ms]
    xo = [torch.empty(n, dtype=torch.complex64, device=dev) for n in npix]
    b.bind(xs, vis, xo, stream)
    for _ in range(args.warmup):
        b.apply(3, stream)
    torch.cuda.synchronize(dev)
    sampler = ClockSampler(0)
    time.sleep(0.5)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    torch.cuda.synchronize(dev)
    w0 = time.time()
    evs[0].record(stream)
    for k in range(args.steps):
        b.apply(3, stream)
        evs[k + 1].record(stream)
    torch.cuda.synchronize(dev)
    w1 = time.time()
    time.sleep(0.3)
    sampler.stop()
    clocks = sampler.summary(sampler.window(w0 - 0.25, w1 + 0.25)) or sampler.summary(sampler.rows)
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = evs[0].elapsed_time(evs[-1]) / args.steps
    # grouped gridding launches alone (same kernels as inside the step)
    t_deg = b.time(8, 10)
    t_grd = b.time(16, 10)
    t_fwd = b.time(1, 10)
    t_adj = b.time(2, 10)
    s8 = 8
    NuNv = [4 * n for n in npix]
    alg_deg = sum(m * (16 + 2 * s8) for m in Ms) + s8 * sum(NuNv)
    peak, peak_kind = measured_peak()
    kern, dur = ("degrid", t_deg) if t_deg >= t_grd else ("grid", t_grd)
    b_step = sum(2 * m * (16 + 2 * s8) for m in Ms) + s8 * sum(7 * g + 3 * n
                                                               for g, n in zip(NuNv, npix))
    out = {
        "metric": "batched degrid+grid Mvis/s (Phi then Phi^H of every channel per step), FP32",
        "value": Mtot / (ms * 1e-3) / 1e6, "unit": "Mvis/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded (PCG64)",
        "config": {"workload": BATCH_WORKLOAD, "channels": len(chans),
                   "visibilities": Mtot, "pixels": int(sum(npix)),
                   "sizes": {str(n): int(sum(1 for c in chans if c["imsizex"] == n))
                             for n in (256, 512, 1024)},
                   "l2": "inputs larger than L2 (%.0f MB of coverage state and visibilities "
                         "per step)" % (Mtot * 24 / 1e6)},
        "tuning": tuning, "latency_ms": {"p50": float(np.percentile(per_step, 50)),
                                         "p99": float(np.percentile(per_step, 99))},
        "stage_ms": {"forward": t_fwd, "adjoint": t_adj, "degrid_launch": t_deg,
                     "grid_launch": t_grd},
        "create_s": t_create, "generate_s": t_gen, "power_method_s": t_power,
        "power_iters": args.power_iters, "device_bytes": info["device_bytes"],
        # own kernels per step: per grid size a row and a column pass each way
        # (3 sizes), degrid, the gather, grid, fold
        "gpu_launches": (4 * info["size_groups"] + 4) * args.steps, "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": kern, "algorithmic_bytes": alg_deg,
                     "achieved": alg_deg / (dur * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": alg_deg / (dur * 1e-3) / 1e9 / peak, "peak_source": peak_kind,
                     "traffic": None},
        "step_roofline": {"algorithmic_bytes": b_step,
                          "achieved_gbs": b_step / (ms * 1e-3) / 1e9,
                          "frac": b_step / (ms * 1e-3) / 1e9 / peak},
    }
    # the same work as single-channel applies, one channel after another
    ops = [pgb.MeasurementOperator(c["u"], c["v"], None, None, c["imsizey"], c["imsizex"], 2.0,
                                   power_iters=0, kernel="kb", Ju=4, Jv=4, precision="fp32")
           for c in chans]
    for op, nrm in zip(ops, norms):
        op.set_norm(float(nrm))
    vis1 = [torch.empty_like(t) for t in vis]
    xo1 = [torch.empty_like(t) for t in xo]

    def seq_step():
        for k, op in enumerate(ops):
            op.forward_into(xs[k], vis1[k], stream)
            op.adjoint_into(vis1[k], xo1[k], stream)
    for _ in range(max(1, args.warmup)):
        seq_step()
    ks = max(3, args.steps // 5)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(ks):
        seq_step()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    ms_seq = e0.elapsed_time(e1) / ks
    b.apply(3, stream)
    torch.cuda.synchronize(dev)
    err_v = max(rel_l2(vis[k].cpu().numpy(), vis1[k].cpu().numpy()) for k in range(len(chans)))
    err_x = max(rel_l2(xo[k].cpu().numpy(), xo1[k].cpu().numpy()) for k in range(len(chans)))
    out["sequential_single_channel"] = {
        "value": Mtot / (ms_seq * 1e-3) / 1e6, "ms_per_step": ms_seq,
        "speedup_batch_over_sequential": ms_seq / ms,
        "max_rel_l2_batch_vs_single": {"forward": err_v, "adjoint": err_x}}
    del ops, vis1, xo1
    # FP64 batch: same channels, same tuning
    if not args.no_fp64:
        b64 = pgb.Batch(chans, J=4, precision="fp64", tuning=tuning)
        b64.set_norms(norms)
        xs64 = [torch.from_numpy(c["x"]).to(dev) for c in chans]
        vis64 = [torch.empty(m, dtype=torch.complex128, device=dev) for m in Ms]
        xo64 = [torch.empty(n, dtype=torch.complex128, device=dev) for n in npix]
        b64.bind(xs64, vis64, xo64, stream)
        for _ in range(max(1, args.warmup)):
            b64.apply(3, stream)
        k64 = max(3, args.steps // 5)
        e0.record(stream)
        for _ in range(k64):
            b64.apply(3, stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms64 = e0.elapsed_time(e1) / k64
        b.apply(3, stream)
        torch.cuda.synchronize(dev)
        fwd_err = max(rel_l2(vis[k].cpu().numpy(), vis64[k].cpu().numpy())
                      for k in range(len(chans)))
        adj_err = max(rel_l2(xo[k].cpu().numpy(), xo64[k].cpu().numpy())
                      for k in range(len(chans)))
        out["fp64"] = {"value": Mtot / (ms64 * 1e-3) / 1e6, "ms_per_step": ms64,
                       "speedup_fp32_over_fp64": ms64 / ms}
        out["rel_l2_fp32_vs_fp64_max_channel"] = {"forward": fwd_err, "adjoint": adj_err}
        del b64, xs64, vis64, xo64
    # end to end: pinned host images in, visibilities and adjoint images out
    if args.e2e_steps > 0:
        xh = [x.cpu().pin_memory() for x in xs]
        vh = [torch.empty(m, dtype=torch.complex64).pin_memory() for m in Ms]
        xoh = [torch.empty(n, dtype=torch.complex64).pin_memory() for n in npix]

        def e2e_step():
            for k in range(len(chans)):
                xs[k].copy_(xh[k], non_blocking=True)
            b.apply(3, stream)
            for k in range(len(chans)):
                vh[k].copy_(vis[k], non_blocking=True)
                xoh[k].copy_(xo[k], non_blocking=True)
            torch.cuda.synchronize(dev)
        e2e_step()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        t_e2e = (time.perf_counter() - t0) / args.e2e_steps
        out["e2e"] = {"value": Mtot / t_e2e / 1e6, "unit": "Mvis/s", "ms_per_step": t_e2e * 1e3,
                      "h2d_bytes_per_step": 8 * int(sum(npix)),
                      "d2h_bytes_per_step": 8 * (Mtot + int(sum(npix))),
                      "api": "Batch.bind once + Batch.apply(3) per step, c64 pinned host copies"}
    if not args.no_cpu_baseline:
        # FP64 oracle: fixed cost (pad + FFT + crop) per image size, per-visibility
        # cost from a sample of the largest channel, summed over the channels
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            fixed = {}
            for n in sorted({c["imsizex"] for c in chans}):
                op0 = oracle.Operator(np.zeros(0), np.zeros(0), None, None, n, n, 2.0,
                                      kernel="kb", Ju=4, Jv=4)
                x0 = synthetic.sky_image(n, n)
                t0 = time.perf_counter()
                op0.adjoint(op0.forward(x0))
                fixed[n] = time.perf_counter() - t0
            big = int(np.argmax(Ms))
            c = chans[big]
            Msmp = min(args.cpu_sample, Ms[big])
            ops_ = oracle.Operator(c["u"][:Msmp], c["v"][:Msmp], None, None, c["imsizey"],
                                   c["imsizex"], 2.0, kernel="kb", Ju=4, Jv=4)
            t0 = time.perf_counter()
            ops_.adjoint(ops_.forward(c["x"]))
            t_s = time.perf_counter() - t0
            per_vis = max(t_s - fixed[c["imsizex"]], 0.0) / Msmp
            t_full = sum(fixed[ch["imsizex"]] for ch in chans) + per_vis * Mtot
            out["cpu_baseline"] = {
                "value": Mtot / t_full / 1e6, "unit": "Mvis/s", "cores": oracle.get_threads(),
                "kind": "port",
                "sample": "FP64 oracle: pad+FFT+crop timed once per image size with M=0, "
                          "per-visibility cost from %d visibilities of channel %d; summed over "
                          "the %d channels" % (Msmp, big, len(chans))}
        except Exception as e:
            out["cpu_baseline"] = {"error": str(e)}
    print(json.dumps(out), flush=True)


SERVE_WORKLOAD = ("Poisson request stream: 70% forward+adjoint, 25% adjoint-only, 5% norm "
                  "(50 power-method rounds); 16 resident coverages, image {256,512,1024}^2, "
                  "M log-uniform in [1e4, 5e6], 70% Gaussian core + 30% uniform, KB J=4")


def serve_stream(pgb, covs, precision, args, t_arr, kinds, cov_idx, xs, vs):
    """Runs the request stream on a fresh server; returns per-request results,
    the server statistics and the wall time of the timed part."""
    srv = pgb.Server(device=0, slots=args.slots, hbm_budget=int(args.budget_gb * (1 << 30)))
    t0 = time.perf_counter()
    ids = [srv.add_coverage(c["u"], c["v"], None, None, c["imsizey"], c["imsizex"],
                            power_iters=10, precision=precision) for c in covs]
    t_setup = time.perf_counter() - t0
    # warm-up: one request of each kind on every coverage
    for k in ids:
        for kind in ("forward_adjoint", "adjoint"):
            srv.wait(srv.submit(k, kind, xs[k], vs[k]))
    srv.wait(srv.submit(ids[0], "norm", iters=5))
    base = srv.stats()
    tickets = [None] * len(t_arr)

    def producer():
        start = time.perf_counter()
        for r in range(len(t_arr)):
            delay = start + t_arr[r] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            c = int(cov_idx[r])
            tickets[r] = srv.submit(ids[c], str(kinds[r]), xs[c], vs[c], iters=50, tol=0.0)
    w0 = time.perf_counter()
    th = threading.Thread(target=producer)
    th.start()
    results = []
    for r in range(len(t_arr)):
        while tickets[r] is None:
            time.sleep(0.0002)
        res = srv.wait(tickets[r])
        if r >= 48:  # outputs of the first requests are kept for the FP32/FP64 comparison
            res.pop("vis", None)
            res.pop("x", None)
        results.append(res)
    th.join()
    wall = time.perf_counter() - w0
    st = srv.stats()
    srv.close()
    return results, st, base, wall, t_setup


def run_serve(args):
    """Request serving: a Poisson stream of forward+adjoint, adjoint-only and
    norm requests on 16 resident coverages; latency from submit to the end of
    the request's device work."""
    import purify_gb300 as pgb
    from purify_gb300 import synthetic
    pgb.build()
    covs = synthetic.config_serve_pool(16, seed=0)
    t_arr, kinds, cov_idx = synthetic.request_stream(args.requests, args.rate, len(covs), seed=1)
    xs = [synthetic.sky_image(c["imsizey"], c["imsizex"], seed=k) for k, c in enumerate(covs)]
    vs = [synthetic.random_vis(c["u"].size, seed=100 + k) for k, c in enumerate(covs)]
    out = None
    per_prec = {}
    clocks = {}
    for prec in (["fp32"] if args.no_fp64 else ["fp32", "fp64"]):
        sampler = ClockSampler(0)
        w0 = time.time()
        res, st, base, wall, t_setup = serve_stream(pgb, covs, prec, args, t_arr, kinds, cov_idx,
                                                    xs, vs)
        w1 = time.time()
        sampler.stop()
        # the timed stream is the last `wall` seconds of the call
        clocks[prec] = (sampler.summary(sampler.window(w1 - wall - 0.25, w1 + 0.25)) or
                        sampler.summary(sampler.rows))
        lat = np.array([r["latency_ms"] for r in res])
        ok = sum(1 for r in res if r["status"] == 0)
        passes = st["visibility_passes"] - base["visibility_passes"]
        by_kind = {}
        for kind in ("forward_adjoint", "adjoint", "norm"):
            sel = [r["latency_ms"] for r, k in zip(res, kinds) if str(k) == kind]
            if sel:
                by_kind[kind] = {"n": len(sel), "p50": float(np.percentile(sel, 50)),
                                 "p99": float(np.percentile(sel, 99))}
        per_prec[prec] = {
            "value": passes / 2 / wall / 1e6, "requests_ok": ok, "wall_s": wall,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "mean": float(lat.mean()), "by_kind": by_kind},
            "queue_ms_p99": float(np.percentile([r["queue_ms"] for r in res], 99)),
            "inflight_peak": st["inflight_peak"], "bytes_peak": st["bytes_peak"],
            "setup_s": t_setup}
        per_prec[prec]["_res"] = res
    f32 = per_prec["fp32"]
    out = {
        "metric": "served degrid+grid Mvis/s and p50/p99 request latency (Poisson stream), FP32",
        "value": f32["value"], "unit": "Mvis/s", "n_gpus": 1, "steps": args.requests,
        "warmup": 33, "ms_per_step": f32["wall_s"] * 1e3 / args.requests,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded (PCG64)",
        "config": {"workload": SERVE_WORKLOAD, "rate_per_s": args.rate, "requests": args.requests,
                   "slots": args.slots, "hbm_budget_gb": args.budget_gb,
                   "latency": "submit to end of the request's device work (D2H included)"},
        "clocks": clocks.get("fp32"), "clocks_fp64": clocks.get("fp64"),
        "latency_ms": f32["latency_ms"], "serving": {k: {kk: vv for kk, vv in v.items()
                                                          if kk != "_res"}
                                                      for k, v in per_prec.items()},
        # own kernels per request (FP32, KB J = 4): the conversions from and
        # to c128, the forward row and column passes and degrid, and grid
        # (gathering caller order), fold and the inverse column and row
        # passes; a norm request: the fill, then per round both FFT
        # directions, the one-pass normal kernel, fold, two reduction kernels
        # and the scale
        "gpu_launches": int(sum({"forward_adjoint": 10, "adjoint": 6}.get(str(k), 1 + 9 * 50)
                                for k in kinds)),
    }
    if "fp64" in per_prec:
        r32, r64 = per_prec["fp32"]["_res"], per_prec["fp64"]["_res"]
        ef = [rel_l2(a["vis"], b["vis"]) for a, b in zip(r32, r64) if "vis" in a]
        ea = [rel_l2(a["x"], b["x"]) for a, b in zip(r32, r64) if "x" in a]
        en = [abs(a["norm"] - b["norm"]) / b["norm"] for a, b in zip(r32, r64)
              if a["norm"] and b["norm"]]
        out["rel_l2_fp32_vs_fp64_max_request"] = {"forward": max(ef) if ef else None,
                                                 "adjoint": max(ea) if ea else None,
                                                 "norm_rel": max(en) if en else None}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.workload == "serve" and args.impl == "gb300":
        run_serve(args)
    elif args.workload == "batch" and args.impl == "gb300":
        run_batch(args)
    elif args.workload == "wproj" and args.impl == "gb300":
        run_wproj(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
