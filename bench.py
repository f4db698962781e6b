"""Benchmark: cell-steps/s of batched OK(+variance)/SK/IDW on one GB300.

Workload (the reference's batched uneven-size configuration, synthetic and
seeded): 1000 stations uniform in a 250 km x 250 km box, 365 daily steps,
each station missing per step with a per-station probability ~ U(0.1, 0.4)
(so 600-900 stations per step); per-step variograms of type Sph / Exp / Gau,
range U(10, 80) km, sill U(0.5, 2), nugget fraction U(0, 0.2); values a
zero-inflated gamma transform (wet fraction 0.6, shape 0.8) of a Gaussian
random field; a 1000 x 1000 grid at 250 m. Methods: OK estimate + variance,
SK estimate, IDW (exponent 2). The 365 steps are cut into 5 slices of 73
steps; one bench step = one slice (slices rotate, so five bench steps cover
the year); a cell-step = one cell at one time step with all three methods.

value: device-resident inputs, timed with CUDA events over K executions.
e2e: the public API call (numpy in, numpy fields out), host<->device copies
inside the timed region. cpu_baseline / --impl reference: the oracle (a
CPU restatement of the reference's own algorithm, incl. its per-cell loop)
on a bounded sample of the same workload, over all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-steps/s for OK/EDK/IDW at <=1e-5 rel err vs FP64; mixed vs plain GPU"
UNIT = "cell-steps/s"
SEED = 20261203
WORKLOAD = "batched_ok_sk_idw_1000stn_365steps_1000x1000"


def make_workload(seed=SEED, n_stns=1000, n_steps=365, nx=1000, ny=1000, cell=250.0,
                  box=250e3):
    from scipy.stats import gamma, norm
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(0, box, n_stns), rng.uniform(0, box, n_stns)
    d = np.hypot(sx[:, None] - sx[None], sy[:, None] - sy[None])
    cov = np.exp(-3 * d / 30e3) + 1e-8 * np.eye(n_stns)
    grf = (np.linalg.cholesky(cov) @ rng.standard_normal((n_stns, n_steps))).T
    u = norm.cdf(grf)
    wet = u > 0.4
    vals = np.where(wet, gamma.ppf(np.clip((u - 0.4) / 0.6, 1e-12, 1 - 1e-12), 0.8, scale=2.0),
                    0.0)
    p_miss = rng.uniform(0.1, 0.4, n_stns)
    vals[rng.uniform(size=(n_steps, n_stns)) < p_miss[None]] = np.nan
    types = np.array(["Sph", "Exp", "Gau"])
    vgs = []
    for j in range(n_steps):
        t = types[rng.integers(3)]
        r = rng.uniform(10e3, 80e3)
        s = rng.uniform(0.5, 2.0)
        nf = rng.uniform(0.0, 0.2)
        vgs.append(f"{nf * s:.5f} Nug(0.0) + {s - nf * s:.5f} {t}({r:.1f})")
    xs = cell / 2 + cell * np.arange(nx)
    ys = box - cell / 2 - cell * np.arange(ny)
    gx, gy = np.meshgrid(xs, ys)
    return dict(sx=sx, sy=sy, z=vals, cx=gx.ravel().copy(), cy=gy.ravel().copy(), vgs=vgs)


def make_small_workload(seed=20261206, n_stns=150, n_steps=24, nx=200, ny=200, cell=500.0,
                        box=100e3):
    """The small configuration: 150 stations uniform in a 100 km box (seeded
    float64 metre coordinates), 24 steps with every station present, values
    5 + a Gaussian random field with the variogram '0.05 Nug(0.0) + 0.95
    Exp(20000)' drawn by Cholesky of the station covariance, a 200 x 200
    grid at 500 m (cell centres, rows from the top)."""
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(0, box, n_stns), rng.uniform(0, box, n_stns)
    d = np.hypot(sx[:, None] - sx[None], sy[:, None] - sy[None])
    cov = 0.95 * np.exp(-3 * d / 20000.0) + 0.05 * np.eye(n_stns)
    vals = 5.0 + (np.linalg.cholesky(cov) @ rng.standard_normal((n_stns, n_steps))).T
    xs = cell / 2 + cell * np.arange(nx)
    ys = box - cell / 2 - cell * np.arange(ny)
    gx, gy = np.meshgrid(xs, ys)
    return dict(sx=sx, sy=sy, z=vals, cx=gx.ravel().copy(), cy=gy.ravel().copy(),
                vgs=["0.05 Nug(0.0) + 0.95 Exp(20000)"] * n_steps)


def _small_cpu_worker(args):
    os.environ["OMP_NUM_THREADS"] = "1"
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["MKL_NUM_THREADS"] = "1"
    sx, sy, z, cx, cy, vgs, iargs = args
    from oracle import port
    t0 = time.perf_counter()
    f, _ = port.interp_steps(sx, sy, z, cx, cy, vgs, iargs, est_vars=True, min_vg_val=1e-4,
                             intrp_dtype=np.float64)
    return time.perf_counter() - t0, f


def small_leg(args, reps=20):
    """The small configuration (150 stations, 24 steps, 200 x 200 cells, OK
    estimate + variance and IDW p=2), where launch overhead matters: the
    whole job per execution, plain FP64 and mixed, eager (one host call per
    kernel) and replayed from a captured CUDA graph, after the cell-tile
    autotuner; e2e through interp_steps; the oracle over all host cores on
    the whole job (cells split across workers), with the GPU's error
    against it."""
    import multiprocessing as mp
    import torch
    import spinterps_gb300 as spi
    from spinterps_gb300.steps import InterpPlan, interp_args_for
    w = make_small_workload()
    iargs = interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float32)
    T, C = w["z"].shape[0], w["cx"].size
    out = {"config": {"workload": "small_ok_idw_150stn_24steps_200x200", "stations": 150,
                      "steps": T, "cells": C, "methods": ["OK+var", "IDW p=2"],
                      "vg": w["vgs"][0]}}

    def per_exec(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    for prec in ("fp64", "mixed"):
        plan = InterpPlan(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], w["vgs"], iargs,
                          precision=prec, **kw)
        plan.execute()
        torch.cuda.synchronize()
        ms_default = per_exec(plan.execute)
        tiles = plan.autotune()
        ms_eager = per_exec(plan.execute)
        plan.capture()
        ms_graph = per_exec(plan.replay)
        out[prec] = {"eager_ms": ms_eager, "graph_ms": ms_graph,
                     "untuned_eager_ms": ms_default,
                     "value_eager": T * C / (ms_eager / 1e3),
                     "value_graph": T * C / (ms_graph / 1e3), "unit": UNIT,
                     "tiles": {f"{k[0]}:{k[2][0]}{k[2][1]}": v for k, v in tiles.items()},
                     "gpu_launches": plan.launches_per_execute()}
        if prec == "fp64":
            f64 = plan.fields()
    e2e = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        spi.interp_steps(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], w["vgs"], iargs, **kw)
        torch.cuda.synchronize()
        e2e.append((time.perf_counter() - t0) * 1e3)
    out["e2e"] = {"value": T * C / (np.median(e2e) / 1e3), "unit": UNIT,
                  "ms": float(np.median(e2e)), "statistic": "median of 3 interp_steps calls",
                  "h2d_bytes_per_step": int(w["z"].nbytes + 16 * (150 + C)),
                  "d2h_bytes_per_step": int(4 * 3 * T * C)}
    if not args.no_cpu:
        cores = os.cpu_count()
        blocks = np.array_split(np.arange(C), cores)
        jobs = [(w["sx"], w["sy"], w["z"], w["cx"][b], w["cy"][b], w["vgs"], iargs)
                for b in blocks]
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(_small_cpu_worker, jobs, chunksize=1)
        wall = time.perf_counter() - t0
        ref = {lab: np.concatenate([r[1][lab] for r in res], axis=1) for lab in res[0][1]}
        errs = {}
        for lab in ref:
            sc = float(np.nanmax(np.abs(ref[lab])))
            errs[lab] = float(np.nanmax(np.abs(f64[lab].astype(np.float64) - ref[lab])) / sc)
        out["cpu_baseline"] = {"value": T * C / wall, "unit": UNIT, "cores": cores,
                               "kind": "port", "cpu_model": cpu_model(), "seed": 20261206,
                               "sample": f"the whole job ({T} steps x {C} cells, OK+var and "
                                         f"IDW p=2), cells split over {cores} workers, wall "
                                         f"{wall:.1f} s (pool start-up included)"}
        out["fp64_err_vs_oracle"] = {"max_rel_to_field_max": errs,
                                     "note": "float32 fields against the oracle's float64"}
    return out


def interp_args():
    from spinterps_gb300.steps import interp_args_for
    return interp_args_for(["OK", "SK", ("IDW", 2.0)], est_vars=True)


KW = dict(est_vars=True, min_var_thr=0.0, min_var_cut=0.0, max_var_cut=None, min_vg_val=1e-4)


# ---------------------------------------------------------------- CPU side
def _cpu_worker(args):
    """One worker of the CPU baseline: the oracle on one step of the workload
    over two cell samples (BLAS pinned to one thread, as the reference's
    driver does). Returns the two wall times."""
    os.environ["OMP_NUM_THREADS"] = "1"
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["MKL_NUM_THREADS"] = "1"
    sx, sy, z, cx, cy, vgs, iargs, sizes = args
    from oracle import port
    out = []
    for c in sizes:
        t0 = time.perf_counter()
        port.interp_steps(sx, sy, z, cx[:c], cy[:c], vgs, iargs, **KW)
        out.append(time.perf_counter() - t0)
    return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    import platform
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def cpu_baseline(w, sizes=(512, 4096), cores=None, step0=0):
    """The oracle (the reference's algorithm, its per-cell pinv loop
    included) over all host cores, one step per worker process, each step
    run on two cell samples of the workload's grid. Per worker the step's
    fixed cost a (station matrices, the two pinv SVDs of OK and SK) and its
    per-cell cost b are fitted from the two timings, and a whole step of the
    workload's C cells costs a + b C: throughput = cores C / mean(a + b C).
    The system solves are thus spread over all C cells, as in a real run."""
    import multiprocessing as mp
    cores = cores or os.cpu_count()
    iargs = interp_args()
    jobs = []
    C = w["cx"].size
    T = w["z"].shape[0]
    steps = [(step0 + k * 37) % T for k in range(cores)]
    for k, st in enumerate(steps):
        # a contiguous block of the grid (rows of cells), spread over workers
        c0 = (k * 7919 * max(sizes)) % (C - max(sizes))
        sl = slice(c0, c0 + max(sizes))
        jobs.append((w["sx"], w["sy"], w["z"][[st]], w["cx"][sl], w["cy"][sl],
                     [w["vgs"][st]], iargs, tuple(sizes)))
    ctx = mp.get_context("spawn")
    # one BLAS thread per worker process (the reference's driver does the
    # same, interp/main.py:31-33); set before the children import numpy
    saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS",
                                             "MKL_NUM_THREADS")}
    for k in saved:
        os.environ[k] = "1"
    try:
        t0 = time.perf_counter()
        with ctx.Pool(cores) as pool:
            res = pool.map(_cpu_worker, jobs, chunksize=1)
        wall = time.perf_counter() - t0
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    c1, c2 = sizes
    b = np.array([max((t2 - t1) / (c2 - c1), 0.0) for t1, t2 in res])
    a = np.array([max(t1 - bb * c1, 0.0) for (t1, _), bb in zip(res, b)])
    t_step = a + b * C
    value = cores * C / float(np.mean(t_step))
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "cpu_model": cpu_model(), "seed": SEED,
            "sample": f"{cores} workers, one step each (steps {steps[0]}, {steps[1]}, ...), "
                      f"each run on {c1} and {c2} cells of the grid (OK+var, SK, IDW p=2; the "
                      f"oracle restating the reference's per-cell pinv loop); per step a fixed "
                      f"cost a (mean {np.mean(a):.2f} s: station matrices and the OK and SK "
                      f"pinv) and a per-cell cost b (mean {np.mean(b) * 1e3:.3f} ms) fitted per "
                      f"worker, extrapolated to the workload's {C} cells per step: "
                      f"cores * C / mean(a + b C); wall {wall:.1f} s",
            "fixed_s_per_step": float(np.mean(a)), "ms_per_cell": float(np.mean(b) * 1e3)}


# ---------------------------------------------------------------- clocks
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, idx=0):
        self.idx = idx
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    return 1900.0, 6800.0, "fallback"


# ---------------------------------------------------------------- GPU side
# The cell kernels' ceilings: the measured peaks for HBM and the
# bf16 tensor pipe; the CUDA-core FP32 / FP64 FMA rates measured here
# (fma_peak_tflops).
KERNEL_BOUND = {
    "var_tc": ("tensor", "spi::k_var_tc (tcgen05 TF32 OK-variance contraction, 5 MMAs per product)"),
    "var_df": ("fp32", "spi::k_var_df (double-float OK-variance contraction, FP32 pipe)"),
    "cells_fp32": ("fp32", "spi::k_krige_cells<float> (FP32 tier: estimates, sum check)"),
    "cells_fp64": ("fp64", "spi::k_krige_cells<double> (FP64 tier: ill-conditioned and "
                           "routed systems, the plain path's kernel)"),
    "idw": ("fp32", "spi::k_idw (FP64 path) / spi::k_idw_tc (mixed path: tcgen05 masked GEMM "
                    "pair)"),
}


_FMA_PEAKS = {}


def fma_peak_tflops(f64):
    """CUDA-core FMA throughput measured on this GPU (spi_peak_fma: 8
    independent chains per thread, 16 CTAs of 256 threads per SM, timed
    with CUDA events; best of 3 after a warm-up launch). MEASURED_PEAKS.json
    covers HBM and the bf16 tensor pipe only."""
    import ctypes
    import torch
    from spinterps_gb300 import _native as nat
    if f64 in _FMA_PEAKS:
        return _FMA_PEAKS[f64]
    sink = torch.empty(152 * 16 * 256, dtype=torch.float64 if f64 else torch.float32,
                       device="cuda")
    thr = ctypes.c_int64(0)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    iters = 20000 if f64 else 200000
    best = 0.0
    for rep in range(4):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        nat.call("spi_peak_fma", 1 if f64 else 0, iters, ctypes.c_void_p(sink.data_ptr()),
                 ctypes.byref(thr), st)
        b.record()
        torch.cuda.synchronize()
        if rep:
            best = max(best, 2 * 8 * iters * thr.value / (a.elapsed_time(b) / 1e3) / 1e12)
    _FMA_PEAKS[f64] = best
    return best


def roofline_for(name, k):
    bf16, hbm, src = measured_peaks()
    bound, kernel = KERNEL_BOUND[name]
    if bound == "tensor":
        peak, psrc = bf16, src + " (bf16 dense; the kernel runs 5 TF32 MMAs per product: a0b0 + a0b1 + a1b0 + a0b2 + a1b1)"
    elif bound == "fp64":
        peak, psrc = fma_peak_tflops(True), "measured FP64 FMA rate (spi_peak_fma, bench.py)"
    else:
        peak, psrc = fma_peak_tflops(False), "measured FP32 FMA rate (spi_peak_fma, bench.py)"
    a = k["achieved_tflops"]
    return {"bound": bound, "kernel": kernel, "achieved": a, "peak": peak, "unit": "TFLOP/s",
            "frac": a / peak, "traffic": None, "peak_source": psrc,
            "per_launch_ms": k["ms"] / max(1, k["launches"]),
            "note": "algorithmic FLOP: per (system, cell) the OK variance n(n+1) and the dual "
                    "columns 2na, per cell-step 2n (right-hand-side generation not counted)"}


def max_over_ranks(ms, world, device):
    """The slowest rank's time: every rank passes its own timed milliseconds
    (replicas, one per GPU); the job's time is their maximum."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_ours(args):
    import torch
    import torch.distributed as dist
    import spinterps_gb300 as spi
    from spinterps_gb300.steps import InterpPlan

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    w = make_workload()
    # replicas: every rank runs its own copy of the workload (the path
    # shards by steps with no exchange; one job per GPU here)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(w)
    iargs = interp_args()
    T_all, C = w["z"].shape[0], w["cx"].size
    n_sl = args.slices
    bounds = np.linspace(0, T_all, n_sl + 1).astype(int)
    plans = []
    for k in range(n_sl):
        sl = slice(bounds[k], bounds[k + 1])
        plans.append(InterpPlan(w["sx"], w["sy"], w["z"][sl], w["cx"], w["cy"], w["vgs"][sl],
                                iargs, precision=args.precision, **KW))
    T = int(np.diff(bounds).max())
    for i in range(args.warmup):
        plans[i % n_sl].execute()
    torch.cuda.synchronize()
    # the cell-tile autotuner on the warmed slices (its choices are cached
    # per station-count bucket and reused by the other slices)
    warmed = {i % n_sl for i in range(args.warmup)}
    tiles = {}
    for k in sorted(warmed):
        tiles.update({f"slice{k}:{kk[0]}:{kk[2][0]}{kk[2][1]}": v
                      for kk, v in plans[k].autotune().items()})
    for k in range(n_sl):
        if k not in warmed:
            plans[k].autotune(cached_only=True)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kev = []
    cell_steps = 0
    with Clocks(local) as clk:
        start.record(stream)
        for i in range(args.steps):
            p = plans[(args.warmup + i) % n_sl]
            kev.append((p, p.execute(timing=True)))
            cell_steps += p.T * C
        end.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    # tier statistics of every slice (after the timed region: slices not yet
    # run there run once more, untimed, so that their probes have decided)
    ran = {i % n_sl for i in range(args.warmup + args.steps)}
    for k in range(n_sl):
        if k not in ran:
            plans[k].execute()
    torch.cuda.synchronize()
    failed = routed = 0
    fp32_steps, df_steps, probe, fp64_why = {}, {}, {}, {}
    for p in plans:
        inf = p.collect_info()
        failed += len(inf["failed_steps"].get("OK", []))
        routed += len(inf.get("exact_inverse_steps", {}).get("OK", []))
        for k, v in inf.get("fp32_tier_steps", {}).items():
            fp32_steps[k] = fp32_steps.get(k, 0) + len(v)
        for k, v in inf.get("df_variance_steps", {}).items():
            df_steps[k] = df_steps.get(k, 0) + len(v)
        # why the OK steps outside the FP32 tiers stay in FP64
        fast_ok = set(inf.get("fp32_tier_steps", {}).get("OK", []))
        rt1 = set(inf.get("exact_inverse_steps", {}).get("OK", []))
        for j, c in inf.get("cond", {}).get("OK", {}).items():
            if j in fast_ok:
                continue
            why = ("exact_inverse" if j in rt1 else
                   "cond_above_cap" if c > p.cond_df else "probe")
            fp64_why[why] = fp64_why.get(why, 0) + 1
        for k, d in inf.get("probe_disc", {}).items():
            probe.setdefault(k, []).append(d)
    ms = max_over_ranks(ms, world, "cuda")
    value = world * cell_steps / (ms / 1e3)
    # per-kernel times (CUDA events on the launching stream) and algorithmic
    # FLOP; the roofline line describes the kernel that takes the most time
    times = {}
    for p, ev in kev:
        for k, (t_ms, n_l, fl) in p.kernel_times(ev).items():
            t = times.setdefault(k, [0.0, 0, 0.0])
            t[0] += t_ms
            t[1] += n_l
            t[2] += fl
    # this library's kernels in the timed region: each timed execution's own count
    launches = sum(plans[(args.warmup + i) % n_sl].launches_per_execute()
                   for i in range(args.steps))
    kernels = {k: {"ms": v[0], "launches": v[1], "achieved_tflops": v[2] / (v[0] / 1e3) / 1e12}
               for k, v in times.items() if v[0] > 0}
    dom_k = max(kernels, key=lambda k: kernels[k]["ms"])
    roofline = roofline_for(dom_k, kernels[dom_k])
    roofline_tc = roofline_for("var_tc", kernels["var_tc"]) if "var_tc" in kernels else None
    idw_ms = times.get("idw", [0.0])[0]
    # e2e: public API from host arrays, fields copied back
    e2e_ms = []
    sl = slice(bounds[0], bounds[1])
    Te = bounds[1] - bounds[0]
    h2d = (w["z"][sl].nbytes + w["sx"].nbytes * 2 + w["cx"].nbytes * 2)
    d2h = 4 * Te * C * len(iargs)
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        spi.interp_steps(w["sx"], w["sy"], w["z"][sl], w["cx"], w["cy"], w["vgs"][sl], iargs,
                         precision=args.precision, **KW)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_val = world * Te * C / (np.median(e2e_ms) / 1e3) if e2e_ms else None
    # plain FP64 GPU path on a step subset, and the mixed path's error on it
    fp64 = None
    if args.fp64_steps > 0 and rank == 0:
        sub = np.arange(args.fp64_steps) * (T // args.fp64_steps)
        zz = w["z"][sub]
        vv = [w["vgs"][s] for s in sub]
        p64 = InterpPlan(w["sx"], w["sy"], zz, w["cx"], w["cy"], vv, iargs, precision="fp64",
                         **KW)
        p64.execute()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        p64.execute()
        b.record()
        torch.cuda.synchronize()
        f64 = p64.fields(numpy=False)
        pm = InterpPlan(w["sx"], w["sy"], zz, w["cx"], w["cy"], vv, iargs, precision="mixed",
                        **KW)
        pm.execute()
        fm = pm.fields(numpy=False)
        errs = {lab: field_errors(fm[lab], f64[lab]) for lab in f64}
        fp64 = {"value": len(sub) * C / (a.elapsed_time(b) / 1e3), "unit": UNIT,
                "sample": f"{len(sub)} evenly spaced steps, all cells",
                "mixed_err_vs_fp64": errs,
                "error_definition": "max / rms: |mixed - fp64| over the field's largest "
                                    "magnitude; per_cell: |mixed - fp64| / |fp64| over cells "
                                    "above the stated floor"}
        del p64, pm
    # variogram fitting of the workload's steps: plain vs learned warm start
    fit = None
    if rank == 0 and not args.no_fit:
        fit = fit_leg(args)
    # the small configuration (150 stations, 24 steps, 200 x 200 cells):
    # launch overhead, CUDA graph, tile autotuner
    small = None
    if rank == 0 and not args.no_small:
        small = small_leg(args)
    # the largest configuration (4000 stations, EDK with two drifts, 2000 x
    # 2000 cells, learned variograms), one wave of its steps
    large = None
    if rank == 0 and not args.no_large:
        del plans
        torch.cuda.empty_cache()
        large = large_leg(args, args.large_reps, fp64_every=args.large_fp64_every, e2e=True,
                          clocks=False)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded; shapes and distributions of the reference's batched "
                    "configuration)",
            "config": {"workload": WORKLOAD, "stations": 1000, "steps": T_all,
                       "steps_per_bench_step": T, "cells": C,
                       "methods": ["OK+var", "SK", "IDW p=2"], "precision": args.precision,
                       "parallelism": f"replicas x{world}",
                       "cell_tiles_autotuned": tiles,
                       "l2": "per-step working set (4.4 GB of fields + 1.6 GB factors) >> L2",
                       "singular_steps_nnb": failed, "exact_inverse_steps": routed,
                       "fp32_tier_steps": fp32_steps,
                       "df_variance_steps": df_steps,
                       "ok_fp64_tier_reasons": fp64_why,
                       "probe_disc_quantiles": {
                           k: {lab: [float(q) for q in np.nanquantile(
                               np.concatenate(v)[:, c], [0.25, 0.5, 0.75, 0.9])]
                               for c, lab in ((0, "est"), (1, "var_tc"), (2, "var_df"))}
                           for k, v in probe.items()}},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "ms": float(np.median(e2e_ms)) if e2e_ms else None,
                    "repeats_ms": [float(x) for x in e2e_ms],
                    "statistic": f"median of {len(e2e_ms)} calls"},
            "gpu_launches": launches,
            "roofline": roofline,
            "roofline_tensor_kernel": roofline_tc,
            "kernels": kernels,
            "idw_ms_per_step": idw_ms / args.steps,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
            "fp64_path": fp64,
            "small": small,
            "large": large,
            "fit": fit,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_profile_case(args):
    """The small case that ncu full captures use: 8 steps of the workload
    (two Exp, two Sph, four Gau from short to long range; two of them take
    the exact-inverse path) over the first 2^17 cells, one execution."""
    import torch
    from spinterps_gb300.steps import InterpPlan
    w = make_workload()
    pick = [2, 3, 0, 7, 308, 142, 29, 271]
    C = 1 << 17
    plan = InterpPlan(w["sx"], w["sy"], w["z"][pick], w["cx"][:C], w["cy"][:C],
                      [w["vgs"][j] for j in pick], interp_args(), precision=args.precision, **KW)
    plan.execute()
    torch.cuda.synchronize()
    print("profile case done")


def _cpu_fit_worker(args):
    os.environ["OMP_NUM_THREADS"] = "1"
    x, y, z, seed = args
    from oracle import fitter
    t0 = time.perf_counter()
    fitter.fit(x, y, z, seed=seed)
    return time.perf_counter() - t0


def fit_leg(args):
    """Variogram fitting of the workload's 365 steps (the reference's fitvgs
    settings): plain GPU fit, warm-started GPU fit, CPU oracle sample, and
    the leave-one-out kriging RMSE of the fitted variograms."""
    import multiprocessing as mp
    import torch
    from spinterps_gb300 import fitvgs, steps, warmstart
    w = make_workload()
    pts = fitvgs.step_points(w["sx"], w["sy"], w["z"])
    T = len(pts)
    cpu = None
    if not args.no_cpu:
        cores = os.cpu_count()
        jobs = [(pts[k][0], pts[k][1], pts[k][2], k) for k in range(cores)]
        ctx = mp.get_context("spawn")
        saved = os.environ.get("OPENBLAS_NUM_THREADS")
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        t0 = time.perf_counter()
        with ctx.Pool(cores) as pool:
            secs = pool.map(_cpu_fit_worker, jobs, chunksize=1)
        wall = time.perf_counter() - t0
        if saved is None:
            os.environ.pop("OPENBLAS_NUM_THREADS", None)
        cpu = {"value": cores / wall, "unit": "fits/s", "cores": cores, "kind": "port",
               "sample": f"{cores} steps, one per core (oracle fitter: the reference's "
                         f"algorithm with scipy DE), median {np.median(secs):.1f} s per fit"}
    mlp = warmstart.WarmStartMLP.load()
    for _ in range(args.warmup):
        fitvgs.fit_steps(None, None, None, emp=fitvgs.Empirical(None, None, None,
                                                                points=pts[:8]).run())
        warmstart.warm_fit_steps(None, None, None, mlp, points=pts[:8])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain, dp = fitvgs.fit_steps(None, None, None, emp=fitvgs.Empirical(
        None, None, None, points=pts).run(), seed=1, return_details=True)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    warm, dw = warmstart.warm_fit_steps(None, None, None, mlp, points=pts, seed=1)
    torch.cuda.synchronize()
    t_warm = time.perf_counter() - t0
    vg_p = [s[-1] if s else "1.0 Nug(0.0)" for s in plain]
    vg_w = [s[-1] if s else "1.0 Nug(0.0)" for s in warm]
    _, r_p = steps.krige_loo(w["sx"], w["sy"], w["z"], vg_p, min_vg_val=1e-4)
    _, r_w = steps.krige_loo(w["sx"], w["sy"], w["z"], vg_w, min_vg_val=1e-4)
    ok = np.isfinite(r_p) & np.isfinite(r_w)
    line = {"metric": "variogram fits/s, learned warm start vs plain fit", "value": T / t_warm,
            "unit": "fits/s", "n_gpus": 1, "higher_is_better": True, "data": "synthetic",
            "config": {"workload": WORKLOAD + "_fit", "steps": T, "fitter": "mdr 0.7, nk 50, "
                       "perm_r_list [1, 2], Sph/Exp + Nug, robust, DE tol 0.01"},
            "plain": {"fits_per_s": T / t_plain, "de_ms": dp["_de_ms"],
                      "de_member_evals": dp["_de_member_evals"]},
            "warm": {"fits_per_s": T / t_warm, "de_ms": dw["_de_ms"],
                     "de_member_evals": dw["_de_member_evals"],
                     "fallback_steps": len(dw["_fallback_steps"]), "ms": dw["_ms"]},
            "speedup_wall": t_plain / t_warm,
            "speedup_de_work": dp["_de_member_evals"] / max(1, dw["_de_member_evals"]),
            "loo_cv_rmse": {"plain": float(r_p[ok].mean()), "warm": float(r_w[ok].mean()),
                            "ratio": float(r_w[ok].mean() / r_p[ok].mean()),
                            "steps": int(ok.sum())},
            "cpu_baseline": cpu}
    return line


def run_fit(args):
    """The fitting leg alone, as its own JSON line."""
    print(json.dumps(fit_leg(args)))


def field_errors(x, y, floor_frac=1e-3):
    """Errors of field x against the FP64 field y (torch tensors, NaN =
    no value): max and RMS of |x - y| relative to y's largest magnitude,
    and per-cell relative errors |x - y| / |y| over the cells with |y| at
    least floor_frac of that magnitude."""
    import torch
    x, y = x.double(), y.double()
    m = torch.isfinite(y)
    sc = y[m].abs().max()
    d = (x[m] - y[m]).abs()
    yy = y[m].abs()
    big = yy >= floor_frac * sc
    rel = d[big] / yy[big]
    return {"max": float(d.max() / sc), "rms": float(d.pow(2).mean().sqrt() / sc),
            "per_cell": {"floor": f"|y| >= {floor_frac:g} x max|y|", "cells": int(big.sum()),
                         "max": float(rel.max()) if rel.numel() else None,
                         "rms": float(rel.pow(2).mean().sqrt()) if rel.numel() else None}}


def refinement_summary(info, kind):
    """The FP32 factor + FP64 refinement path of a plan's ``collect_info``:
    steps refined over the FP32 factor, steps whose refinement did not
    converge (solved again over an FP64 factor), and the correction counts
    of the refined steps."""
    its = list(info.get("ir_iters", {}).get(kind, {}).values())
    return {"steps": len(info.get("ir_steps", {}).get(kind, [])),
            "fp64_fallback_steps": len(info.get("ir_fallback_steps", {}).get(kind, [])),
            "iterations": ({"min": int(min(its)), "median": float(np.median(its)),
                            "max": int(max(its))} if its else None)}


def large_leg(args, reps, fp64_every=1, e2e=False, clocks=True):
    """The large hourly EDK configuration on one wave of steps: 4000
    stations in a 500 km box, per-station missingness U(0.05, 0.5), two
    drifts (fBm elevation, easting), a 2000 x 2000 grid at 250 m, float32
    fields; each step's variogram from the learned warm start with cold-fit
    fallback (timed apart). The mixed path runs the whole wave ``reps``
    times; the plain FP64 path runs every ``fp64_every``-th step of it once
    (both rates are per cell-step: every step has its own system), and the
    mixed fields of those steps are compared with it."""
    import torch
    from spinterps_gb300 import fitvgs, synth, warmstart
    import spinterps_gb300 as spi
    from spinterps_gb300.steps import InterpPlan
    from spinterps_gb300.steps import interp_args_for
    T = args.large_steps
    t0 = time.perf_counter()
    w = synth.large_edk(n_steps=T, nx=args.large_nx, ny=args.large_nx,
                        device="cpu" if args.synth_cpu else "cuda")
    t_gen = time.perf_counter() - t0
    pts = fitvgs.step_points(w["sx"], w["sy"], w["z"])
    mlp = warmstart.WarmStartMLP.load()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    strs, det = warmstart.warm_fit_steps(None, None, None, mlp, points=pts, seed=1)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    vgs = [s[-1] if s else "1.0 Nug(0.0)" for s in strs]
    iargs = interp_args_for(["EDK"], est_vars=False)
    C = w["cx"].size
    kw = dict(stn_drifts=w["stn_drift"], cell_drifts=w["cell_drift"], min_vg_val=1e-4,
              intrp_dtype=np.float32, arena_budget=96 << 30)

    def timed(plan, n):
        evs, tot = [], []
        for _ in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            ev = plan.execute(timing=True)
            b.record()
            torch.cuda.synchronize()
            tot.append(a.elapsed_time(b))
            evs.append(ev)
        times = {}
        for ev in evs:
            for k, (t_ms, n_l, fl) in plan.kernel_times(ev).items():
                t = times.setdefault(k, [0.0, 0, 0.0])
                t[0] += t_ms
                t[1] += n_l
                t[2] += fl
        return float(np.median(tot)), tot, times

    pm = InterpPlan(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], vgs, iargs, precision="mixed",
                    **kw)
    pm.execute()
    clk = Clocks(0) if clocks else None
    if clk:
        clk.__enter__()
    ms_m, all_m, times_m = timed(pm, reps)
    if clk:
        clk.__exit__()
    launches = pm.launches_per_execute()
    info = pm.collect_info()
    cond = np.array(list(info["cond"]["EDK"].values()))
    n_fast = len(info.get("fp32_tier_steps", {}).get("EDK", []))
    n_cap = int(np.sum(cond <= pm.cond_split))
    refinement = refinement_summary(info, "EDK")
    failed = sorted(info.get("failed_steps", {}).get("EDK", []))
    sub = np.arange(0, T, fp64_every)
    fm = pm.flds["EDK"][torch.as_tensor(sub, device=pm.flds["EDK"].device)].clone()
    del pm
    torch.cuda.empty_cache()
    err = fp64 = None
    if not args.skip_fp64:
        p64 = InterpPlan(w["sx"], w["sy"], w["z"][sub], w["cx"], w["cy"], [vgs[i] for i in sub],
                         iargs, precision="fp64", **kw)
        ms_64, _, times_64 = timed(p64, 1)
        err = field_errors(fm, p64.flds["EDK"])
        fp64 = {"value": len(sub) * C / (ms_64 / 1e3), "unit": UNIT, "ms": ms_64,
                "sample": f"every {fp64_every}th step of the wave ({len(sub)} steps), all cells",
                "kernels_ms": {k: v[0] for k, v in times_64.items()}}
        del p64
        torch.cuda.empty_cache()
    e2e_val = None
    if e2e:
        zh = np.asarray(w["z"].cpu().numpy() if hasattr(w["z"], "cpu") else w["z"])
        host = {k: (v.cpu().numpy() if hasattr(v, "cpu") else np.asarray(v))
                for k, v in w.items() if k in ("sx", "sy", "cx", "cy", "stn_drift",
                                               "cell_drift")}
        kwh = dict(kw, stn_drifts=host["stn_drift"], cell_drifts=host["cell_drift"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        spi.interp_steps(host["sx"], host["sy"], zh, host["cx"], host["cy"], vgs, iargs,
                         precision="mixed", **kwh)
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3
        e2e_val = {"value": T * C / (e2e_ms / 1e3), "unit": UNIT, "ms": e2e_ms,
                   "h2d_bytes_per_step": int(zh.nbytes + sum(v.nbytes for v in host.values())),
                   "d2h_bytes_per_step": int(4 * T * C)}
    kernels = {k: {"ms": v[0], "launches": v[1], "achieved_tflops": v[2] / (v[0] / 1e3) / 1e12}
               for k, v in times_m.items() if v[0] > 0}
    dom_k = max(kernels, key=lambda k: kernels[k]["ms"])
    n_av = np.isfinite(np.asarray(w["z"].cpu() if hasattr(w["z"], "cpu") else w["z"])).sum(1)
    out = {"value": T * C / (ms_m / 1e3), "unit": UNIT, "ms_per_execution": ms_m,
           "executions_ms": all_m,
           "config": {"workload": f"large_edk_4000stn_{T}of8760steps_{args.large_nx}x"
                                  f"{args.large_nx}", "stations": 4000,
                      "steps": T, "cells": C, "methods": ["EDK (elevation, easting)"],
                      "stations_per_step": [int(n_av.min()), int(n_av.max())],
                      "output": "float32", "vgs": "learned warm start, cold-fit fallback"},
           "fp64_path": fp64,
           "mixed_over_fp64": (T * C / (ms_m / 1e3)) / fp64["value"] if fp64 else None,
           "mixed_err_vs_fp64": err, "e2e": e2e_val, "gpu_launches": launches,
           "kernels": kernels, "roofline": roofline_for(dom_k, kernels[dom_k]),
           "tiers": {"fp32": n_fast, "fp64": int(cond.size - n_fast), "cond_under_cap": n_cap,
                     "cond_median": float(np.median(cond)), "cond_max": float(cond.max())},
           "refinement": refinement,
           # singular systems above the pinv check's size: nearest station
           "singular_steps_nnb": {"count": len(failed), "steps": failed[:8],
                                  "vgs": [vgs[j] for j in failed[:8]]},
           "fit": {"seconds": t_fit, "fallback_steps": len(det["_fallback_steps"]),
                   "de_ms": det["_de_ms"], "ms": det["_ms"]},
           "synthesis_s": t_gen}
    if clk:
        out["clocks"] = clk.summary()
    return out


def run_year(args):
    """The large hourly configuration over its whole year: all 8760 steps
    (4000 stations, EDK with two drifts, 2000 x 2000 cells, float32 fields,
    learned variograms) through the public wave API
    (spinterps_gb300.waves.interp_steps_waves), the steps in waves sized to
    a device budget, every wave's fields copied to host memory and reduced
    there to per-step means by the sink. Wall time of the whole call, host
    planning and copies included."""
    import torch
    from spinterps_gb300 import fitvgs, synth, warmstart, waves
    from spinterps_gb300.steps import interp_args_for
    T = args.year_steps
    t0 = time.perf_counter()
    w = synth.large_edk(n_steps=T, nx=args.large_nx, ny=args.large_nx)
    t_gen = time.perf_counter() - t0
    pts = fitvgs.step_points(w["sx"], w["sy"], w["z"])
    mlp = warmstart.WarmStartMLP.load()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    # the fitter holds every station pair of its steps on the device (~4e6
    # per step here): the year's steps go through it 256 at a time
    strs, fit_fallback = [], 0
    for k in range(0, T, 256):
        sk, det = warmstart.warm_fit_steps(None, None, None, mlp, points=pts[k:k + 256], seed=1)
        strs.extend(sk)
        fit_fallback += len(det["_fallback_steps"])
        torch.cuda.empty_cache()
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    vgs = [s[-1] if s else "1.0 Nug(0.0)" for s in strs]
    iargs = interp_args_for(["EDK"], est_vars=False)
    C = w["cx"].size
    means = np.full(T, np.nan)
    n_waves = [0]

    def sink(first, flds):
        v = flds["EDK"]
        means[first:first + v.shape[0]] = np.nanmean(v[:, ::97], axis=1)
        n_waves[0] += 1

    with Clocks(0) as clk:
        t0 = time.perf_counter()
        prblm, info = waves.interp_steps_waves(
            w["sx"], w["sy"], w["z"], w["cx"], w["cy"], vgs, iargs, sink=sink,
            budget=int(args.year_budget_gb * 2 ** 30), stn_drifts=w["stn_drift"],
            cell_drifts=w["cell_drift"], min_vg_val=1e-4, intrp_dtype=np.float32,
            precision="mixed")
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    fast = sum(len(i["info"].get("fp32_tier_steps", {}).get("EDK", [])) for i in info)
    ir = sum(len(i["info"].get("ir_steps", {}).get("EDK", [])) for i in info)
    iters = [v for i in info for v in i["info"].get("ir_iters", {}).get("EDK", {}).values()]
    line = {"metric": METRIC, "value": T * C / wall, "unit": UNIT, "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"large_edk_4000stn_{T}steps_{args.large_nx}x{args.large_nx}",
                       "stations": 4000, "steps": T, "cells": C, "methods": ["EDK"],
                       "api": "waves.interp_steps_waves, fields to host per wave",
                       "budget_gb": args.year_budget_gb},
            "wall_s": wall, "waves": n_waves[0], "problem_steps": len(prblm),
            "fp32_tier_steps": fast, "ir_steps": ir,
            "ir_iterations": {str(k): int(np.sum(np.asarray(iters) == k))
                              for k in sorted(set(iters))},
            "plan_s": float(sum(i["plan_s"] for i in info)),
            "field_mean_range": [float(np.nanmin(means)), float(np.nanmax(means))],
            "fit_s": t_fit, "fit_fallback_steps": fit_fallback, "synthesis_s": t_gen,
            "clocks": clk.summary()}
    print(json.dumps(line))


def run_large(args):
    """The large configuration alone: its own JSON line (every step through
    both paths)."""
    d = large_leg(args, args.steps, fp64_every=1, e2e=False)
    line = {"metric": METRIC, "value": d["value"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "higher_is_better": True, "dtype": "f32+f64",
            "data": "synthetic (seeded; shapes and distributions of the reference's large hourly "
                    "configuration)"}
    line.update({k: v for k, v in d.items() if k not in ("value", "unit")})
    print(json.dumps(line))


def run_stress(args):
    """The precision-stress EDK configuration: 400 Thomas-clustered stations
    (20 parents, sigma 300 m) in a 100 km box, a Gaussian variogram of range
    30 km with a 1e-6 micro-range nugget, one fBm elevation drift, 200 steps,
    a 500 x 500 grid. Mixed and plain FP64 paths on the same plan inputs; the
    mixed path's error against FP64 and the tiers its probe chose."""
    import torch
    from spinterps_gb300 import synth
    from spinterps_gb300.steps import InterpPlan
    from spinterps_gb300.steps import interp_args_for
    w = synth.stress_edk()
    iargs = interp_args_for(["EDK"], est_vars=False)
    C, T = w["cx"].size, w["z"].shape[0]
    kw = dict(stn_drifts=w["stn_drift"], cell_drifts=w["cell_drift"], intrp_dtype=np.float32)
    res = {}
    for prec in ("mixed", "fp64"):
        p = InterpPlan(w["sx"], w["sy"], w["z"], w["cx"], w["cy"], w["vgs"], iargs,
                       precision=prec, **kw)
        for _ in range(max(1, args.warmup)):
            p.execute()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.steps):
            p.execute()
        b.record()
        torch.cuda.synchronize()
        info = p.collect_info()
        res[prec] = (a.elapsed_time(b) / args.steps, p.flds["EDK"].double(), info)
    f64, fm = res["fp64"][1], res["mixed"][1]
    m = torch.isfinite(f64)
    sc = f64[m].abs().max()
    dd = (fm[m] - f64[m]).abs()
    info = res["mixed"][2]
    cond = np.array(list(info["cond"]["EDK"].values()))
    line = {"metric": METRIC, "value": T * C / (res["mixed"][0] / 1e3), "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "higher_is_better": True, "dtype": "f32+f64",
            "data": "synthetic (seeded; the reference's precision-stress configuration)",
            "config": {"workload": "stress_edk_400stn_thomas_200steps_500x500", "stations": 400,
                       "steps": T, "cells": C, "methods": ["EDK (fBm elevation)"],
                       "variogram": w["vgs"][0]},
            "fp64_path": {"value": T * C / (res["fp64"][0] / 1e3), "unit": UNIT,
                          "ms": res["fp64"][0]},
            "mixed_ms": res["mixed"][0], "mixed_over_fp64": res["fp64"][0] / res["mixed"][0],
            "mixed_err_vs_fp64": {"max": float(dd.max() / sc),
                                  "rms": float(dd.pow(2).mean().sqrt() / sc)},
            "tiers": {"fp32_steps": len(info.get("fp32_tier_steps", {}).get("EDK", [])),
                      "fp64_steps": T - len(info.get("fp32_tier_steps", {}).get("EDK", [])),
                      "cond_min": float(cond.min()), "cond_max": float(cond.max())},
            "refinement": refinement_summary(info, "EDK")}
    print(json.dumps(line))


def run_legacy(args):
    """The single-neighbourhood classes (cyth/interpmthds.pyx:251-765):
    OrdinaryKriging of 400 stations onto the cells of a legacy_nx^2 grid
    (default 500 x 500 = 250 000 output points), with every array the class
    exposes materialised (rhss, lambdas, the inverse). value: the kernels on
    device-resident inputs (spi_legacy_system + spi_legacy_points); e2e: the
    class call, numpy in and numpy out; cpu_baseline: the oracle's
    restatement of the class's per-point loop (np.matmul(pinv, rhs) per
    point, serial like the reference's class) on a sample of points."""
    import torch
    from spinterps_gb300 import legacy
    from oracle import port
    rng = np.random.default_rng(SEED + 7)
    n, nx, box = 400, args.legacy_nx, 1e5
    xi, yi = rng.uniform(0, box, n), rng.uniform(0, box, n)
    zi = rng.gamma(1.2, 3.0, n)
    cs = box / nx
    gx = np.arange(nx) * cs + 0.5 * cs
    cx, cy = np.meshgrid(gx, gx[::-1])
    cx, cy = cx.ravel().copy(), cy.ravel().copy()
    n_out, m = cx.size, n + 1
    model = "0.1 Nug(0.0) + 0.9 Exp(30000)"
    dv = [torch.as_tensor(a, device="cuda") for a in (xi, yi, zi, cx, cy)]
    st = torch.cuda.current_stream()
    for _ in range(max(3, args.warmup)):
        r = legacy.krige_points("OK", *dv, model)
    torch.cuda.synchronize()
    evs = []
    with Clocks() as clk:
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            r = legacy.krige_points("OK", *dv, model)
            e1.record(st)
            evs.append((e0, e1))
        torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
    assert r["route"] == "gj"
    # e2e: the class, numpy in and out (copies inside)
    t0 = time.perf_counter()
    obj = legacy.OrdinaryKriging(xi, yi, zi, cx, cy, model=model)
    obj.krige()
    t_e2e = time.perf_counter() - t0
    h2d = 8 * (3 * n + 2 * n_out)
    d2h = 8 * (n * n + 2 * m * m + n_out * m + n_out * n + 3 * n_out)
    # the oracle on a bounded sample of points, timed on one host core
    samp = min(n_out, args.legacy_cpu_points)
    sel = rng.choice(n_out, samp, replace=False)
    t0 = time.perf_counter()
    ref = port.legacy_krige("OrdinaryKriging", xi, yi, zi, cx[sel], cy[sel], model)
    t_cpu = time.perf_counter() - t0
    err = float(np.abs(obj.zk[sel] - ref["zk"]).max() / np.abs(ref["zk"]).max())
    flop = 2.0 * m * m * n_out
    bf16, hbm, src = measured_peaks()
    line = {"metric": "legacy_points_per_s", "value": n_out / (ms / 1e3), "unit": "points/s",
            "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"legacy_ordinary_kriging_{n}stn_{nx}x{nx}",
                       "stations": n, "points": n_out, "variogram": model,
                       "l2": "outputs (1.6 GB per step) exceed L2"},
            "e2e": {"value": n_out / t_e2e, "unit": "points/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": 4 * args.steps,
            "roofline": {"bound": "fp64", "kernel": "spi::k_leg_lambda (lambda = P r, FP64)",
                         "achieved": flop / (ms / 1e3) / 1e12, "peak": fma_peak_tflops(True),
                         "unit": "TFLOP/s",
                         "frac": flop / (ms / 1e3) / 1e12 / fma_peak_tflops(True),
                         "traffic": None,
                         "peak_source": "measured FP64 FMA rate (spi_peak_fma, bench.py)",
                         "note": "2 m^2 FLOP per point over the whole step time (the "
                                 "factorisation, right-hand sides and epilogue count "
                                 "against it)"},
            "cpu_baseline": {"value": samp / t_cpu, "unit": "points/s", "cores": 1,
                             "kind": "port", "sample": f"{samp} random points of the grid, "
                             "the per-point loop of the reference's class"},
            "err_vs_oracle": err, "clocks": clk.summary()}
    print(json.dumps(line))


def run_nebs(args):
    """The neighbour methods (interp/steps.py:584-833): the batched
    workload's stations and first steps, OK+var / IDW from each cell's 16
    nearest present stations ('nrst') on a nebs_nx^2 grid. value: through
    interp_steps (spi_neb_select, spi_local_groups for kriging,
    spi_local_cells for IDW): wall time of the whole call, numpy in and
    out, its host work per step group included; entries_ms: device time per
    entry point in a second run;
    cpu_baseline: the oracle's restatement (the reference's per-group loop)
    on a sample."""
    import torch
    import spinterps_gb300 as spi
    from oracle import port
    w = make_workload()
    T, nx = args.nebs_steps, args.nebs_nx
    box = 250e3
    g = (np.arange(nx) + 0.5) * (box / nx)
    cx, cy = np.meshgrid(g, g[::-1])
    cx, cy = cx.ravel().copy(), cy.ravel().copy()
    z, vgs = w["z"][:T], w["vgs"][:T]
    from spinterps_gb300.steps import interp_args_for
    iargs = interp_args_for(["OK", ("IDW", 2.0)], est_vars=True)
    kw = dict(est_vars=True, min_vg_val=1e-4, intrp_dtype=np.float32, neb_sel_mthd="nrst",
              n_nebs=16, n_pies=1)
    spi.interp_steps(w["sx"], w["sy"], z[:2], cx[:1000], cy[:1000], vgs[:2], iargs, **kw)
    torch.cuda.synchronize()
    with Clocks() as clk:
        t0 = time.perf_counter()
        out, _ = spi.interp_steps(w["sx"], w["sy"], z, cx, cy, vgs, iargs, **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    # a second run with each native call bracketed by CUDA events on its
    # stream: device time per entry point
    from spinterps_gb300 import _native as nat
    spans, plain_call = {}, nat.call

    def timed_call(name, *a):
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        rc = plain_call(name, *a)
        e1.record(s)
        spans.setdefault(name, []).append((e0, e1))
        return rc

    nat.call = timed_call
    try:
        spi.interp_steps(w["sx"], w["sy"], z, cx, cy, vgs, iargs, **kw)
        torch.cuda.synchronize()
    finally:
        nat.call = plain_call
    entries = {k: {"ms": sum(a.elapsed_time(b) for a, b in v), "calls": len(v)}
               for k, v in spans.items()}
    C = cx.size
    # the oracle on a small block of cells and steps
    rng = np.random.default_rng(5)
    sel = rng.choice(C, args.nebs_cpu_cells, replace=False)
    ts = 2
    t0 = time.perf_counter()
    ref, _ = port.interp_steps(w["sx"], w["sy"], z[:ts], cx[sel], cy[sel], vgs[:ts], iargs,
                               **kw)
    t_cpu = time.perf_counter() - t0
    got, _ = spi.interp_steps(w["sx"], w["sy"], z[:ts], cx[sel], cy[sel], vgs[:ts], iargs, **kw)
    err = {lab: float(np.nanmax(np.abs(got[lab] - ref[lab])) / np.nanmax(np.abs(ref[lab])))
           for lab in ref}
    line = {"metric": "cell-steps/s, neighbour method nrst (16), OK+var and IDW",
            "value": T * C / dt, "unit": "cell-steps/s", "n_gpus": 1, "steps": 1,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"nebs_nrst16_1000stn_{T}steps_{nx}x{nx}", "stations": 1000,
                       "steps": T, "cells": C, "methods": ["OK+var", "IDW p=2"]},
            "seconds": dt,
            "cpu_baseline": {"value": ts * sel.size / t_cpu, "unit": "cell-steps/s",
                             "cores": 1, "kind": "port",
                             "sample": f"{sel.size} random cells x {ts} steps, the oracle's "
                                       "per-group loop"},
            "err_vs_oracle_on_sample": err, "entries_ms": entries, "clocks": clk.summary()}
    print(json.dumps(line))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    w = make_workload()
    vals = []
    for i in range(args.warmup + args.steps):
        # each bench step: one pool over all host cores, a different step
        # of the workload per worker (about 5 s)
        vals.append(cpu_baseline(w, step0=i))
    timed = vals[args.warmup:]
    v = float(np.median([x["value"] for x in timed]))
    cb = dict(timed[0])
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "stations": int(w["sx"].size),
                       "steps": int(w["z"].shape[0]), "cells": int(w["cx"].size),
                       "methods": ["OK+var", "SK", "IDW p=2"]},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-large", action="store_true",
                    help="leave the large configuration out of the default line")
    ap.add_argument("--year", action="store_true",
                    help="the large configuration over all its steps through the wave API")
    ap.add_argument("--year-steps", type=int, default=8760)
    ap.add_argument("--year-budget-gb", type=float, default=24.0)
    ap.add_argument("--no-fit", action="store_true",
                    help="leave variogram fitting out of the default line")
    ap.add_argument("--no-small", action="store_true",
                    help="leave the small configuration out of the default line")
    ap.add_argument("--small", action="store_true",
                    help="the small configuration alone (CUDA graph and autotuner)")
    ap.add_argument("--large-reps", type=int, default=2)
    ap.add_argument("--large-fp64-every", type=int, default=4)
    ap.add_argument("--fp64-steps", type=int, default=4)
    ap.add_argument("--slices", type=int, default=5)
    ap.add_argument("--fit", action="store_true",
                    help="variogram fitting benchmark (plain vs learned warm start)")
    ap.add_argument("--profile-case", action="store_true",
                    help="run the small case used for ncu full captures and exit")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--large", action="store_true",
                    help="the large hourly EDK configuration (one wave of steps) instead")
    ap.add_argument("--large-steps", type=int, default=152)
    ap.add_argument("--large-nx", type=int, default=2000,
                    help="grid side of the large configuration (2000 = the configuration's)")
    ap.add_argument("--synth-cpu", action="store_true",
                    help="with --large: synthesise the fields on the CPU")
    ap.add_argument("--skip-fp64", action="store_true",
                    help="with --large: skip the plain FP64 comparison (profiling runs)")
    ap.add_argument("--stress", action="store_true",
                    help="the precision-stress EDK configuration instead")
    ap.add_argument("--legacy", action="store_true",
                    help="the single-neighbourhood OrdinaryKriging class instead")
    ap.add_argument("--legacy-nx", type=int, default=500)
    ap.add_argument("--legacy-cpu-points", type=int, default=4000)
    ap.add_argument("--nebs", action="store_true",
                    help="the neighbour method 'nrst' (one kriging system per neighbour group) instead")
    ap.add_argument("--nebs-nx", type=int, default=500)
    ap.add_argument("--nebs-steps", type=int, default=73)
    ap.add_argument("--nebs-cpu-cells", type=int, default=2000)
    args = ap.parse_args()
    if args.small:
        print(json.dumps(dict(small_leg(args), metric=METRIC, unit=UNIT, n_gpus=1)))
        return
    if args.year:
        run_year(args)
        return
    if args.nebs:
        run_nebs(args)
    elif args.legacy:
        run_legacy(args)
    elif args.profile_case:
        run_profile_case(args)
    elif args.fit:
        run_fit(args)
    elif args.large:
        run_large(args)
    elif args.stress:
        run_stress(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
