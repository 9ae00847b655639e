"""Benchmark: statistic + gradient evaluations per second on the C2 workload.

Workload (synthetic, seeded): 1024x1024 Sersic + Exponential + FlatSky, 63x63
Moffat PSF, central 40x40 region oversampled 5x with a 315x315 PSF, 10% random
mask, Poisson noise, chi^2 with data-based errors, 12 free parameters.  One
"step" = one fit statistic plus its full gradient for one parameter vector
(what one Levenberg-Marquardt iteration needs).

Arms
  gb300 (default):
    value  -- fast path (FP32 evaluation and FFTs, FP64 setup and reductions,
              adjoint gradient), parameter vector already in device memory,
              one CUDA-graph launch per step, timed with CUDA events on the
              library's stream; L2 is flushed (256 MiB write) before each step.
    e2e    -- the same through the host C-ABI call imfit_GetFitStatisticAndGradient
              with pinned host buffers: parameters copied in, statistic and
              gradient copied out, every step.
    plain_fp64_fd -- the drop-in FP64 path with a forward-difference gradient
              (1 + 12 model evaluations per step, mpfit's step rule), same GPU.
    cpu_baseline -- the CPU port of the reference path (oracle/), all host cores.
  reference (--impl reference):
    the reference's algorithm on the host CPU (the oracle port; the reference's
    own build needs its checkout, which the GPU host does not have), same metric.
Multi-GPU (torchrun): independent replicas, one per GPU, no collective on the data
path; value = sum over ranks (weak scaling).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "statistic+gradient evals/s vs plain FP64 + FD Jacobian, same GPU, <=1e-5 rel err"
UNIT = "evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--cpu-units", type=int, default=3, help="statistic+gradient units in the CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", default="C2", choices=["C1", "C2", "C3", "C4", "C5"])
    ap.add_argument("--batch", type=int, default=0,
                    help="C4: evaluate only the first N of the 256 parameter vectors (small profiling cases)")
    ap.add_argument("--c5-count", type=int, default=4096, help="cutouts in the C5 batch")
    ap.add_argument("--c5-threads", type=int, default=8, help="host threads driving the C5 size buckets")
    ap.add_argument("--c5-mode", default="set", choices=["set", "buckets"],
                    help="C5: one cutout set (one launch per stage) or size buckets of image stacks")
    ap.add_argument("--c5-check", type=int, default=12, help="C5 cutouts re-fitted in FP64 on the CPU")
    ap.add_argument("--no-graphs", action="store_true", help="launch kernels one by one (for profilers)")
    ap.add_argument("--jtwj", action="store_true",
                    help="time the forward-mode normal equations (J^T W J, J^T W dev) instead of the gradient")
    ap.add_argument("--fft-plan", default=None, metavar="CAND,ORDER",
                    help="pin the FFT plan (padded-length candidate, radix order) instead of autotuning it; "
                         "profiling runs use the plan a timed run reported (launch_shape.pin)")
    ap.add_argument("--launch-shape", default=None, metavar="RPB,THREADS,CPB,CTHREADS",
                    help="pin the launch shape (rows per CTA, row threads, columns per CTA, column threads)")
    return ap.parse_args()


def apply_pins(m, args):
    """Fixed FFT plan / launch shape from the command line (profiling runs:
    under a profiler the autotuner's timings, and so its choices, differ)."""
    if args.fft_plan:
        c, o = (int(v) for v in args.fft_plan.split(","))
        m.set_fft_plan(c, o)
    if args.launch_shape:
        r, t, c, ct = (int(v) for v in args.launch_shape.split(","))
        m.set_launch_shape(r, t, c, ct)


def measured_profile(config, stage):
    """ncu figures of a stage from the committed summary: DRAM bytes per launch
    and SM / issue utilisation (or None)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_per_launch.json")) as f:
            return json.load(f).get(config, {}).get(stage)
    except (OSError, ValueError):
        return None


def measured_traffic(config, stage):
    """DRAM bytes per launch of a stage from the committed ncu summary (or None)."""
    v = measured_profile(config, stage)
    return float(v["dram_bytes"]) if v else None


def max_over_ranks(value, world):
    """Largest value over the ranks (replicas are timed separately; the job
    takes as long as its slowest rank).  gloo on the host, no GPU collective."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def workload(name, batch=0):
    from imfit_gb300 import workloads
    wl = {"C1": workloads.c1, "C2": workloads.c2, "C3": workloads.c3, "C4": workloads.c4}[name]()
    if batch and wl.batch is not None:
        wl.batch = wl.batch[:batch]
    return wl


def config_block(wl, extra=None):
    cfg = {"workload": f"{wl.name}: {wl.ncols}x{wl.nrows}, " + "+".join(f for f, _ in wl.functions)
           + (f", PSF {wl.psf.shape[1]}x{wl.psf.shape[0]}" if wl.psf is not None else "")
           + "".join(f", region {r[2]} x{r[1]} PSF {r[0].shape[0]}" for r in wl.regions)
           + f", {wl.stat}", "n_params": wl.n_params,
           "batch_per_step": 1 if wl.batch is None else len(wl.batch),
           "l2": "flushed (256 MiB write) before every timed step"}
    if extra:
        cfg.update(extra)
    return cfg


# ------------------------------------------------------------------ CPU arm
CPU_WHAT = ("the project's C restatement of the reference's path (oracle/imfit_oracle.c: the reference's "
            "ModelObject/Convolver/FunctionObject arithmetic, OpenMP over pixels), with the project's own FP64 "
            "FFT on 7-smooth padded sizes standing in for FFTW; neither the reference's sources nor FFTW are "
            "on the GPU host")


def cpu_time(wl, units, threads=None):
    """Time `units` statistic+gradient units (1 + n_params evaluations each) of
    the CPU port with all host threads (or `threads`); returns (units/s, threads)."""
    import oracle
    oracle.build_restatement()
    m = oracle.OracleModel()
    m.set_fft_smooth(True)
    threads = threads or os.cpu_count() or 1
    m.set_max_threads(threads)
    from imfit_gb300 import workloads
    workloads.configure(m, wl)
    p = np.array(wl.start, dtype=float)
    m.get_fit_statistic(p)  # warm
    eps = np.sqrt(2.2204460e-16)
    t0 = time.perf_counter()
    for _ in range(units):
        m.get_fit_statistic(p)
        for j in range(len(p)):
            q = p.copy()
            q[j] += eps * abs(q[j]) if q[j] != 0 else eps
            m.get_fit_statistic(q)
    dt = time.perf_counter() - t0
    return units / dt, threads


def run_reference(args, rank, world):
    if rank != 0:
        return
    wl = workload(args.config, args.batch)
    import oracle
    from imfit_gb300 import workloads
    workloads.synthesize(wl, oracle.OracleModel)
    for _ in range(args.warmup and 1):
        cpu_time(wl, 1)
    rates = []
    threads = 1
    for _ in range(max(1, min(args.steps, 3))):
        r, threads = cpu_time(wl, 1)
        rates.append(r)
    v = float(np.mean(rates))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(rates), "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": config_block(wl, {"parallelism": "host OpenMP"}),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(rates)} statistic+gradient units of {wl.name} "
                                       f"({wl.n_params + 1} FP64 model evaluations each), FFTs padded to "
                                       f"7-smooth sizes", "what": CPU_WHAT},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
class _Nvml:
    """Read-only NVML queries through the driver's libnvidia-ml (SM clock,
    maximum SM clock, current clock-event reasons) for the device torch
    uses, found by UUID (NVML does not follow CUDA_VISIBLE_DEVICES)."""
    CLOCK_SM = 1  # nvmlClockType_t NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index):
        import ctypes
        import torch
        self.c = ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        uuid = getattr(torch.cuda.get_device_properties(index), "uuid", None)
        st = 1
        if uuid is not None:
            st = lib.nvmlDeviceGetHandleByUUID(("GPU-" + str(uuid)).encode(), ctypes.byref(self.h))
        if st != 0:
            st = lib.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h))
        if st != 0:
            raise OSError("no NVML handle")
        self.lib = lib
        self.reasons = (getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
                        or lib.nvmlDeviceGetCurrentClocksThrottleReasons)

    def sample(self):
        c, r = self.c.c_uint(), self.c.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, self.CLOCK_SM, self.c.byref(c)) != 0:
            return None
        if self.reasons(self.h, self.c.byref(r)) != 0:
            return None
        return float(c.value), [nm for bit, nm in self.REASONS.items() if r.value & bit]

    def max_sm(self):
        c = self.c.c_uint()
        return float(c.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, self.CLOCK_SM, self.c.byref(c)) == 0 \
            else None


class Clocks:
    """SM clock and throttle reasons sampled while the timed region runs:
    NVML from a thread every 2 ms (a timed region of a few tens of ms still
    gets samples), else nvidia-smi's 200 ms loop."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        import threading
        self.proc = None
        self.nvml = None
        self.samples = []
        try:
            self.nvml = _Nvml(index)
        except Exception:  # no driver library, no device, an older NVML: use nvidia-smi
            self.nvml = None
        if self.nvml is not None:
            self.halt = threading.Event()
            first = self.nvml.sample()
            if first:
                self.samples.append(first)
            self.thread = threading.Thread(target=self._loop, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def _loop(self):
        while not self.halt.wait(0.002):
            v = self.nvml.sample()
            if v:
                self.samples.append(v)

    def stop(self):
        if self.nvml is not None:
            self.halt.set()
            self.thread.join()
            last = self.nvml.sample()
            if last:
                self.samples.append(last)
            sm = [c for c, _ in self.samples]
            reasons = sorted({r for _, rs in self.samples for r in rs})
            return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": self.nvml.max_sm(),
                    "reasons": reasons, "samples": len(sm), "source": "nvml"}
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out = self.proc.communicate(timeout=5)[0]
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out = self.proc.communicate()[0]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in out.strip().splitlines():
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


def algorithmic_bytes(model, wl):
    """HBM bytes each fast-path kernel must move per launch (one parameter vector)."""
    from imfit_gb300 import build  # noqa: F401
    # spectrum geometry mirrors the library's choice of 7-smooth padded sizes
    def smooth(n, even):
        m = n
        while True:
            if not (even and m % 2):
                k = m
                for p in (2, 3, 5, 7):
                    while k % p == 0:
                        k //= p
                if k == 1:
                    return m
            m += 1
    P = wl.psf.shape
    N = (wl.nrows, wl.ncols)
    W = (N[0] + P[0] - 1, N[1] + P[1] - 1)
    Lx, Ly = smooth(W[1], True), smooth(W[0], True)
    pitch = Lx // 2 + 1
    c8 = 8  # complex64
    out = {
        "eval_r2c": W[0] * pitch * c8,
        "cols_conv": (W[0] + Ly + N[0]) * pitch * c8,
        "stat_rows": 2 * N[0] * pitch * c8 + N[0] * N[1] * 8,
        "cols_adjoint": (N[0] + Ly + W[0]) * pitch * c8,
        "grad_rows": W[0] * pitch * c8,
        # 3-D line of sight: per window pixel the value and its r~ slope out (eval),
        # r~ in and one partial per CTA out (grad); the kept subinterval lists are
        # scratch whose size depends on the integrands
        "los_eval": W[0] * W[1] * 8,
        "los_grad": W[0] * W[1] * 4,
    }
    if wl.regions:
        psf, k, (x1, x2, y1, y2) = wl.regions[0]
        n = x2 - x1 + 1
        sub = n * k
        rw = sub + psf.shape[0] - 1
        rl = smooth(rw, True)
        rp = rl // 2 + 1
        out.update({"region_eval_r2c": rw * rp * c8, "region_cols_conv": (rw + rl + sub) * rp * c8,
                    "region_down": sub * rp * c8, "region_g_r2c": sub * rp * c8,
                    "region_cols_adjoint": (sub + rl + rw) * rp * c8, "region_grad_rows": rw * rp * c8})
    return out


# ------------------------------------------------- per-unit roofline (B, F)
# transcendental (MUFU) operations of one profile evaluation: Sersic sqrt, lg2,
# ex2, ex2; Exponential sqrt, ex2; GaussianRing sqrt, ex2; Moffat lg2, ex2;
# Gaussian ex2; constant and planar backgrounds none
SFU_PER_EVAL = {"Sersic": 4, "Exponential": 2, "GaussianRing": 2, "Moffat": 2, "Gaussian": 1,
                "FlatSky": 0, "TiltedSkyPlane": 0}
# CalculateSubsamples (func_sersic.cpp, func_exp.cpp, func_moffat.cpp,
# func_gaussian.cpp): (index of the scale parameter in the function's own
# parameters, inner radius with 20 subsamples, small-scale count)
SUB_RULE = {"Sersic": (4, 4.0, 20), "Exponential": (3, 3.0, 20), "Moffat": (3, 3.0, 40), "Gaussian": (3, 3.0, 40)}


def _n_subsamples(kind, scale, r):
    _, rin, small = SUB_RULE[kind]
    ns = np.ones(r.shape, dtype=np.int64)
    near = r < 10.0
    tiny = near & (scale <= 1.0) & (r <= 1.0)
    ns[tiny] = min(100, int(small / scale)) if scale > 0 else 100
    inner = near & ~tiny & (r <= rin)
    ns[inner] = 20
    outer = near & ~tiny & ~inner
    ns[outer] = np.minimum(100, (20.0 / np.maximum(r[outer], 1e-30)).astype(np.int64))
    return np.maximum(ns, 1)


def sfu_ops_per_unit(wl, p):
    """F(U): MUFU operations of one statistic + gradient evaluation at p: every
    window pixel evaluated twice (forward, gradient recompute) and every
    subsample of the pixels within radius 10 once (the precomputed table), on
    the main window and, at k x resolution, on the oversampled region's window.
    None for the 3-D line-of-sight functions (their count depends on the
    adaptive integration)."""
    from imfit_gb300 import workloads
    names = workloads.param_names(wl.functions)
    P = wl.psf.shape[0] if wl.psf is not None else 1
    grids = [(np.arange(1 - P // 2, wl.ncols + P // 2 + 1, dtype=np.float64),
              np.arange(1 - P // 2, wl.nrows + P // 2 + 1, dtype=np.float64))]
    for psf, k, (x1, x2, y1, y2) in wl.regions:
        h = psf.shape[0] // 2
        grids.append((x1 + (0.5 / k - 0.5) + np.arange(-h, (x2 - x1 + 1) * k + h) / k,
                      y1 + (0.5 / k - 0.5) + np.arange(-h, (y2 - y1 + 1) * k + h) / k))
    total = 0
    off = 0
    x0 = y0 = 0.0
    for i, (fn, new_set) in enumerate(wl.functions):
        if new_set or i == 0:
            x0, y0 = p[off], p[off + 1]
            off += 2
        nfp = {"Sersic": 5, "Exponential": 4, "FlatSky": 1, "GaussianRing": 5, "Moffat": 5, "Gaussian": 4,
               "TiltedSkyPlane": 3}.get(fn)
        if nfp is None:
            return None
        fp = p[off:off + nfp]
        off += nfp
        m = SFU_PER_EVAL[fn]
        if m == 0:
            continue
        pa = np.deg2rad(fp[0] + 90.0)
        q = 1.0 - fp[1]
        for xs, ys in grids:
            dx = xs[None, :] - x0
            dy = ys[:, None] - y0
            xp = dx * np.cos(pa) + dy * np.sin(pa)
            yp = (-dx * np.sin(pa) + dy * np.cos(pa)) / q
            r = np.sqrt(xp * xp + yp * yp)
            total += 2 * m * r.size
            if fn in SUB_RULE:
                ns = _n_subsamples(fn, fp[SUB_RULE[fn][0]], r)
                total += m * int(np.sum((ns * ns)[ns > 1]))
    assert off == len(names)
    return int(total)


def survey_bytes_per_unit(wl):
    """B(U) of the per-unit roofline as the survey defines it, on the
    reference's padded grids (N_model = N + 2P, N_pad = N_model + P - 1):
    data and weights in FP32, plus forward and adjoint of one r2c -> column
    pass x PSF -> c2r convolution (5 complex passes + real read and write)
    on the main grid and on each oversampled region."""
    P = wl.psf.shape[0] if wl.psf is not None else 0

    def conv(n_model, p):
        n_pad = n_model + p - 1
        return 2 * (40 * n_pad * (n_pad // 2 + 1) + 8 * n_model * n_model)

    b = wl.ncols * wl.nrows * 8 + (conv(wl.nrows + 2 * P, P) if P else 0)
    for psf, k, (x1, x2, y1, y2) in wl.regions:
        po = psf.shape[0]
        b += conv((x2 - x1 + 1) * k + 2 * po, po)
    return int(b)


def accuracy_vs_oracle(m, wl, P):
    """Fast statistic and plain FP64 statistic of the GPU library against the
    FP64 oracle (oracle/: the reference's algorithm on the reference's padded
    sizes) on the same inputs, for up to four of the step's parameter vectors."""
    import oracle
    from imfit_gb300 import workloads
    oracle.build_restatement()
    o = workloads.configure(oracle.OracleModel(), wl)
    o.set_max_threads(os.cpu_count() or 1)
    fast, plain = [], []
    for p in P[:4]:
        so = o.get_fit_statistic(p)
        fast.append(abs(m.fit_statistic_fast(p) - so) / abs(so))
        plain.append(abs(m.get_fit_statistic(p) - so) / abs(so))
    return {"stat_rel_err_vs_oracle": max(fast), "plain_fp64_stat_rel_err_vs_oracle": max(plain),
            "vectors_checked": len(fast), "oracle": "oracle.OracleModel (FP64 C restatement, reference padding)"}


def run_gpu(args, rank, local_rank, world):
    import torch

    import imfit_gb300
    from imfit_gb300 import build, workloads
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    wl = workload(args.config, args.batch)
    workloads.synthesize(wl, lambda: imfit_gb300.ModelObject(local_rank))
    m = workloads.configure(imfit_gb300.ModelObject(local_rank), wl)
    apply_pins(m, args)
    nP = wl.n_params
    stream = torch.cuda.ExternalStream(m.stream(), device=dev)
    p0 = np.array(wl.start, dtype=np.float64)
    P = np.array(wl.batch if wl.batch is not None else [wl.start], dtype=np.float64)
    B = P.shape[0]

    # accuracy: against the FP64 oracle (the reference's algorithm restated in
    # C, on the reference's own padded FFT sizes) on the same inputs, and
    # against this GPU's plain FP64 path
    accuracy = accuracy_vs_oracle(m, wl, P) if rank == 0 else None
    s64 = m.get_fit_statistic(p0)
    s_fast, g_fast = m.statistic_and_gradient(p0)
    s_fd, g_fd = m.statistic_and_gradient_fd(p0)
    gscale = np.abs(g_fd) + 1e-3 * np.max(np.abs(g_fd))
    gerr = np.abs(g_fast - g_fd) / gscale
    if accuracy is not None:
        accuracy.update({"stat_rel_err_vs_gpu_fp64": abs(s_fast - s64) / abs(s64),
                         "grad_err_vs_gpu_fp64_fd": {"median": float(np.median(gerr)), "max": float(np.max(gerr)),
                                                     "norm": "|g - g_fd| / (|g_fd| + 1e-3 max|g_fd|), "
                                                             "forward differences, subsampling on"}})

    d_params = torch.tensor(P.ravel(), dtype=torch.float64, device=dev)
    d_stat = torch.zeros(B, dtype=torch.float64, device=dev)
    d_grad = torch.zeros(B * nP, dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MiB > 129 MB L2
    m.set_use_graphs(not args.no_graphs)

    def step():
        m.batch_device(B, d_params.data_ptr(), d_stat.data_ptr(), d_grad.data_ptr())

    # calibration (not timed): every kernel bracketed by events, stages serial
    m.set_kernel_timing(True)
    m.set_kernel_timing_stage(None)
    per_kernel = {}
    with torch.cuda.stream(stream):
        for i in range(args.warmup + 10):
            flush.fill_(1.0)
            step()
            kt = m.kernel_times()  # synchronizes the library stream
            if i >= args.warmup:
                for name, ms in kt:
                    per_kernel.setdefault(name, []).append(ms)
    cal = {k: float(np.mean(v)) for k, v in per_kernel.items()}
    dom = max(cal, key=cal.get)
    kernels_per_step = len(cal)

    # timed region: concurrent stages exactly as a caller runs them -- no
    # timing events inside the step (an event between two kernels ends their
    # programmatic-dependent-launch overlap)
    m.set_kernel_timing(False)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            step()
    torch.cuda.synchronize()
    times = []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local_rank)
    # NVTX range "timed_region": lets a profiler restrict its launch list to
    # the timed steps (ncu --clock-control none --nvtx --nvtx-include "timed_region/")
    torch.cuda.nvtx.range_push("timed_region")
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    for a, b in ev:
        times.append(a.elapsed_time(b))
    t_ms = max_over_ranks(float(np.sum(times)), world)
    value = world * B * args.steps / (t_ms / 1e3)

    # the dominant kernel's duration: the same K steps again, concurrent, with
    # events recorded on its stream around that kernel only
    m.set_kernel_timing(True)
    m.set_kernel_timing_stage(dom)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            step()
    torch.cuda.synchronize()
    dom_ms = []
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            step()
            dom_ms += [ms for _, ms in m.kernel_times()]
    torch.cuda.synchronize()
    clk = clocks.stop()
    m.set_kernel_timing(False)

    # end-to-end through the host C ABI, pinned buffers
    import ctypes
    lib = imfit_gb300.load_library()
    hp = ctypes.c_void_p()
    nin, nout = B * nP, B + B * nP
    lib.imfit_HostAlloc(8 * (nin + nout), ctypes.byref(hp))
    hbuf = np.ctypeslib.as_array((ctypes.c_double * (nin + nout)).from_address(hp.value))
    hbuf[:nin] = P.ravel()
    DP = ctypes.POINTER(ctypes.c_double)
    pp = hbuf[:nin].ctypes.data_as(DP)
    ps = hbuf[nin:nin + B].ctypes.data_as(DP)
    pg = hbuf[nin + B:].ctypes.data_as(DP)
    for _ in range(args.warmup):
        lib.imfit_BatchFitStatisticAndGradient(m.h, B, pp, ps, pg)
    e2e_t = 0.0
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = lib.imfit_BatchFitStatisticAndGradient(m.h, B, pp, ps, pg)
        e2e_t += time.perf_counter() - t0
        assert st == 0
    e2e_t = max_over_ranks(e2e_t, world)
    e2e = world * B * args.steps / e2e_t
    lib.imfit_HostFree(hp)

    # plain FP64 + finite-difference gradient (the drop-in), same GPU
    for _ in range(min(2, args.warmup)):
        m.statistic_and_gradient_fd(p0)
    pt = 0.0
    for i in range(args.plain_steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        m.statistic_and_gradient_fd(p0)
        pt += time.perf_counter() - t0
    pt = max_over_ranks(pt, world)
    plain = args.plain_steps / pt

    # roofline of the dominant kernel
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    total = sum(cal.values())
    ab = algorithmic_bytes(m, wl)
    kernel_table = {k: {"ms": round(v, 5), "share": round(v / total, 4),
                        "GBps": round(B * ab[k] / (v * 1e-3) / 1e9, 1) if k in ab and v > 0 else None}
                    for k, v in sorted(cal.items(), key=lambda kv: -kv[1])}
    dom_avg = float(np.mean(dom_ms)) if dom_ms else cal[dom]
    achieved = B * ab.get(dom, 0) / (dom_avg * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
            "frac": round(achieved / hbm_peak, 4), "peak_source": peak_src,
            "algorithmic_bytes_per_launch": B * ab.get(dom, 0), "kernel_ms": round(dom_avg, 5),
            "kernel_ms_how": "CUDA events around the kernel on its stream in a second pass of the K timed steps "
                             "(the headline steps carry no events)",
            "traffic": measured_traffic(args.config, dom)}
    prof = measured_profile(args.config, dom)
    if prof:  # the same kernel's compute-side utilisation (ncu, committed summary)
        roof["ncu"] = {k: prof.get(k) for k in ("sm_pct", "issue_pct", "warps_active_pct", "alu_pct", "fma_pct",
                                                "xu_pct", "dram_pct") if prof.get(k) is not None}
        roof["limiter"] = prof.get("limiter")
    # per-unit roofline T_roof = B / BW_HBM + F / P_SFU (one statistic + gradient
    # evaluation); frac = T_roof x achieved units/s
    try:
        p_sfu = imfit_gb300.measure_sfu_rate(local_rank)
    except Exception:  # measurement helper unavailable: report without it
        p_sfu = None
    F = sfu_ops_per_unit(wl, p0)
    has_los = any(f in ("ExponentialDisk3D", "FerrersBar3D") for f, _ in wl.functions)
    b_path = int(sum(v for k, v in ab.items() if has_los or not k.startswith("los_")))
    b_survey = survey_bytes_per_unit(wl)
    if F is not None and p_sfu:
        t_roof = b_path / (hbm_peak * 1e9) + F / p_sfu
        roof["per_unit"] = {"T_roof_us": round(t_roof * 1e6, 3), "frac": round(t_roof * value / world, 4),
                            "bytes": b_path, "bytes_survey_padding": b_survey,
                            "T_roof_us_survey_padding": round((b_survey / (hbm_peak * 1e9) + F / p_sfu) * 1e6, 3),
                            "sfu_ops": F, "p_sfu_ops_per_s": p_sfu, "bw_gbs": hbm_peak,
                            "bytes_definition": "sum of the fast path's per-kernel algorithmic bytes (FP32 spectra "
                                                "on 7-smooth padded windows) for one unit",
                            "sfu_definition": "2 x window pixels x MUFU ops per profile + subsamples of pixels "
                                              "within radius 10, main window and oversampled region"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, threads = cpu_time(wl, args.cpu_units)
        rate1, _ = cpu_time(wl, 1, threads=1)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "one_thread": {"value": rate1, "unit": UNIT, "cores": 1, "sample": f"1 unit of {wl.name}"},
               "sample": f"{args.cpu_units} statistic+gradient units of {wl.name} "
                         f"({nP + 1} FP64 model evaluations each, forward differences)",
               "what": CPU_WHAT}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 eval / f64 setup+reductions",
                "data": "synthetic (seeded), model-generated with Poisson + read noise",
                "config": config_block(wl, {"parallelism": f"replicas x{world}" if world > 1 else "single GPU"}),
                "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * nin, "d2h_bytes_per_step": 8 * nout},
                "plain_fp64_fd": {"value": plain * world, "unit": UNIT, "steps": args.plain_steps,
                                  "evals_per_step": nP + 1},
                "speedup_vs_plain_fp64_fd": {"device": value / (plain * world), "e2e": e2e / (plain * world)},
                "accuracy": accuracy,
                "roofline": roof, "launch_shape": m.launch_shape(), "kernels_serial_calibration": kernel_table, "gpu_launches": kernels_per_step * args.steps,
                "clocks": clk, "cpu_baseline": cpu}
        print(json.dumps(line), flush=True)


def run_c5(args, rank, local_rank, world):
    """C5: every cutout of an uneven batch fitted by the batched LM (one step =
    all cutouts fitted from their starts).  value = fits/s; accuracy = largest
    parameter difference against FP64 fits (scipy's MINPACK lmdif on the
    oracle's FP64 deviates) of a few cutouts."""
    import torch

    import imfit_gb300
    from imfit_gb300 import build, cutouts, workloads
    build.build()
    torch.cuda.set_device(local_rank)
    items = workloads.c5(args.c5_count, seed=1005 + rank)
    t0 = time.time()
    imgs = workloads.synthesize_c5(items, lambda: imfit_gb300.ModelObject(local_rank))
    t_synth = time.time() - t0
    cs = [cutouts.Cutout(d, s, p) for d, s, p in imgs]
    t0 = time.time()
    fitter = cutouts.CutoutFitter(workloads.C5_FUNCTIONS, cs, device=local_rank, threads=args.c5_threads,
                                  mode=args.c5_mode)
    t_setup = time.time() - t0
    starts = np.array([it["start"] for it in items])
    lo = np.array([it["lower"] for it in items])
    hi = np.array([it["upper"] for it in items])
    for _ in range(max(1, args.warmup)):
        r = fitter.fit(starts, lower=lo, upper=hi, ftol=1e-8)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks = Clocks(local_rank)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = fitter.fit(starts, lower=lo, upper=hi, ftol=1e-8)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    clk = clocks.stop()
    t_fit = max_over_ranks(t_fit, world)
    value = world * len(items) * args.steps / t_fit
    # accuracy against FP64 fits (oracle deviates, scipy's trust-region least
    # squares with the same limits and tight tolerances) of a few cutouts of
    # side <= 120 px spread over the sizes: (1) the FP64 minimum nearest to our
    # fit (the FP64 fit started from our parameters) -- how far our solution
    # is from a true FP64 minimum; (2) the FP64 fit from the same start --
    # whether both optimisers end in the same basin (the model is multimodal:
    # bulge and disk can trade places, ellipticities pin at limits).
    acc = None
    if rank == 0 and args.c5_check > 0:
        import scipy.optimize as so

        import oracle
        oracle.build_restatement()
        small = [i for i in np.argsort([it["side"] for it in items]) if items[i]["side"] <= 120]
        order = [small[int(k)] for k in np.linspace(0, len(small) - 1, min(args.c5_check, len(small)))]
        errs = []
        for i in order:
            d, sg, p = imgs[i]
            o = oracle.OracleModel()
            for name, new_set in workloads.C5_FUNCTIONS:
                o.add_function(name, new_set)
            o.finish_functions()
            o.add_psf(p)
            o.add_image_data(d)
            o.add_error_vector(sg)
            o.final_setup()
            got = r["params"][i]
            fit64 = lambda x0: so.least_squares(lambda x: o.compute_deviates(x), x0, bounds=(lo[i], hi[i]),
                                                method="trf", x_scale="jac", xtol=1e-15, ftol=1e-15, gtol=1e-15,
                                                max_nfev=20000)
            near = fit64(np.clip(got, lo[i], hi[i]))
            same = fit64(starts[i])
            # sigma from the FP64 fit's own Jacobian; parameters held at a limit
            # in either fit (pegged) have no sigma and are reported apart
            sig = np.sqrt(np.abs(np.diag(np.linalg.pinv(near.jac.T @ near.jac))))
            tol_l = 1e-9 * np.maximum(1.0, np.abs(lo[i]))
            tol_h = 1e-9 * np.maximum(1.0, np.abs(hi[i]))
            pegged = ((np.abs(near.x - lo[i]) <= tol_l) | (np.abs(near.x - hi[i]) <= tol_h) |
                      (np.abs(got - lo[i]) <= tol_l) | (np.abs(got - hi[i]) <= tol_h))
            # parameters without effect at the FP64 minimum (a position angle at zero
            # ellipticity): no sigma, reported with the pegged ones
            cn = np.linalg.norm(near.jac, axis=0)
            pegged |= cn <= 1e-9 * np.max(cn)
            chi_got = o.get_fit_statistic(got)
            chi_near, chi_same = float(near.fun @ near.fun), float(same.fun @ same.fun)
            diff = got - near.x
            for j in (2, 7):  # position angles: PA and PA + 180 are the same model
                diff[j] = (diff[j] + 90.0) % 180.0 - 90.0
            relv = np.abs(diff) / np.maximum(np.abs(near.x), 1e-12)
            osv = np.where(sig > 0, np.abs(diff) / np.where(sig > 0, sig, 1.0), np.inf)
            relv = np.where(pegged, 0.0, relv)
            osv = np.where(pegged, 0.0, osv)
            errs.append({"side": int(items[i]["side"]),
                         "pegged_params": int(np.sum(pegged)),
                         "max_rel_err": float(np.max(relv)),
                         "max_err_over_sigma": float(np.max(osv)),
                         "chi2_rel_diff_vs_nearest_fp64": float((chi_got - chi_near) / chi_near),
                         "chi2_rel_diff_vs_same_start_fp64": float((chi_got - chi_same) / chi_same),
                         "rel": relv, "over_sigma": osv})
        rel = np.array([e["rel"] for e in errs])
        osg = np.array([e["over_sigma"] for e in errs])
        same = np.array([e["chi2_rel_diff_vs_same_start_fp64"] for e in errs])
        acc = {"cutouts_checked": int(len(order)),
               "reference": "nearest FP64 minimum: scipy least_squares (trf, same limits, tolerances 1e-15) on the "
                            "oracle's FP64 deviates, started from this fit",
               "pegged_params": int(sum(e["pegged_params"] for e in errs)),
               "note": "parameters at a limit in either fit, or without effect at the FP64 minimum, are excluded "
                       "from the error statistics (pegged_params)",
               "max_param_rel_err": float(rel.max()),
               "max_param_err_over_sigma": float(osg.max()),
               "fraction_params_within_1e-4_rel": float(np.mean(rel <= 1e-4)),
               "fraction_params_within_1e-4_rel_or_0.01_sigma": float(np.mean((rel <= 1e-4) | (osg <= 0.01))),
               "fraction_params_within_1e-4_rel_per_param": [float(v) for v in np.mean(rel <= 1e-4, axis=0)],
               "same_start_fp64": {"fraction_same_chi2_1e-6": float(np.mean(np.abs(same) <= 1e-6)),
                                   "fraction_lower_chi2_here": float(np.mean(same < -1e-6)),
                                   "fraction_higher_chi2_here": float(np.mean(same > 1e-6))},
               "per_cutout": [{k: v for k, v in e.items() if k not in ("rel", "over_sigma")} for e in errs]}
    if rank == 0:
        sides = np.array([it["side"] for it in items])
        line = {"metric": "cutout fits/s (batched LM, forward-mode JtWJ, FP32 eval / FP64 reductions and solve)",
                "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * t_fit / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32 eval / f64 reductions+solve",
                "data": "synthetic (seeded) cutouts: FP64 model + Gaussian noise",
                "config": {"workload": f"C5: {len(items)} cutouts, side {sides.min()}-{sides.max()} px "
                                       f"(mean area {float((sides ** 2).mean()):.0f} px), Sersic+Exponential, "
                                       "Moffat PSF 25-63 px, chi^2",
                           "mode": args.c5_mode + (" (one handle, one launch per stage over all cutouts)"
                                                   if args.c5_mode == "set" else ""),
                           "buckets": len(fitter.buckets), "host_threads": args.c5_threads if fitter.buckets else 1,
                           "parallelism": "single GPU"},
                "lm": {"status_counts": {str(k): int(v) for k, v in zip(*np.unique(r["status"], return_counts=True))},
                       "mean_rounds": float(np.mean(r["niter"])),
                       # last timed fit: J^T W J evaluations (device work + transfers) vs the host's LM steps
                       "timing": fitter.model.lm_batch_stats() if getattr(fitter, "model", None) else None},
                "accuracy": acc, "setup_s": {"synthesize": t_synth, "stacks": t_setup}, "clocks": clk}
        print(json.dumps(line), flush=True)


def run_jtwj(args, rank, local_rank, world):
    """Forward-mode normal equations of the LM path (imfit_BatchJtWJDevice):
    statistic, J^T W J and J^T W dev for the step's parameter vectors; one
    step = one call, L2 flushed before each.  Reported on its own line (not the
    headline metric)."""
    import torch

    import imfit_gb300
    from imfit_gb300 import build, workloads
    build.build()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    wl = workload(args.config, args.batch)
    workloads.synthesize(wl, lambda: imfit_gb300.ModelObject(local_rank))
    m = workloads.configure(imfit_gb300.ModelObject(local_rank), wl)
    apply_pins(m, args)
    nP = wl.n_params
    P = np.array(wl.batch if wl.batch is not None else [wl.start], dtype=np.float64)
    B = P.shape[0]
    stream = torch.cuda.ExternalStream(m.stream(), device=dev)
    d_p = torch.tensor(P.ravel(), dtype=torch.float64, device=dev)
    d_s = torch.zeros(B, dtype=torch.float64, device=dev)
    d_a = torch.zeros(B * nP * nP, dtype=torch.float64, device=dev)
    d_b = torch.zeros(B * nP, dtype=torch.float64, device=dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    m.set_use_graphs(not args.no_graphs)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.fill_(1.0)
            m.batch_jtwj_device(B, d_p.data_ptr(), d_s.data_ptr(), d_a.data_ptr(), d_b.data_ptr())
    torch.cuda.synchronize()
    clocks = Clocks(local_rank)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.nvtx.range_push("timed_region")
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            m.batch_jtwj_device(B, d_p.data_ptr(), d_s.data_ptr(), d_a.data_ptr(), d_b.data_ptr())
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    t_ms = max_over_ranks(float(sum(a.elapsed_time(b) for a, b in ev)), world)
    if rank == 0:
        print(json.dumps({"metric": "forward-mode J^T W J evaluations/s", "value": world * B * args.steps / (t_ms / 1e3),
                          "unit": "evals/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                          "config": config_block(wl), "clocks": clk}), flush=True)


def main():
    args = parse()
    rank, local_rank, world = dist_info()
    if world > 1:
        import torch.distributed as dist
        if args.impl == "reference":
            dist.init_process_group("gloo")
        else:
            import torch
            torch.cuda.set_device(local_rank)
            dist.init_process_group("gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.config == "C5":
        run_c5(args, rank, local_rank, world)
    elif args.jtwj:
        run_jtwj(args, rank, local_rank, world)
    else:
        run_gpu(args, rank, local_rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
