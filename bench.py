"""Benchmark: LM solve seconds to reach <= 1.001x the FP64 reference cost, one GB300.

One step = one full LM solve of the workload's synthetic problem, from the same
initial parameters, until the cost first reaches the target (1.001 x the FP64
reference final cost of this workload) or max_iterations. Metric (lower is
better): seconds per step.

Default workload: 5 (5,000 cameras / 1,500,000 points / 8,788,960 observations,
power-law tracks 2-200, 5% outliers), in the specified chosen form: "learned"
(FP32 Jacobians and implicit FP32 Schur matvecs, PCG with the learned
correction judged by block-Jacobi, FP64 iterative refinement of every Schur
step to a relative residual of 1e-8, inner PCG tolerance 1e-4).

  value  device-resident: the problem is on the device before the timed region;
         each step resets the parameters on the device and runs the LM loop
         (gba_solver_run). CUDA events on the solver stream, synchronize on both
         sides.
  e2e    the reference-facing call gba_solve_bal on pinned host buffers: H2D of
         the problem, setup, the solve and the D2H of the parameters, every step.
Extra keys, each measured in this run:
  inexact_newton       the same solve with inexact Gauss-Newton steps (Schur
                       systems solved to a relative residual of 0.1, the forcing
                       term of Ceres' iterative Schur solver; no refinement)
  plain_fp64_form      the plain all-FP64 form (dense S on the device, DMMA
                       Cholesky): one solve to the same target (--no-plain skips it)
  cpu_pair             the oracle (CPU restatement of the reference LM, all host
                       cores) and this library, both timed to the target on a
                       smaller workload (2 by default) whose CPU solve fits the run
  cpu_baseline         the oracle on a bounded sample of the benchmark workload,
                       scaled to a whole solve (extrapolated, a lower bound)
Inputs (~0.9 GB of observations, ~1 GB of per-slot Jacobians) exceed the
129 MB L2, so no L2 flush is needed between steps.

--impl reference: the CPU arm. It runs the oracle's LM solve (nothing of this
library is loaded: the problem comes from the oracle's own generator) to the
target; when that solve cannot fit the run (the dense 9C x 9C Cholesky on the
host cores, e.g. 45,000^2 at workload 5) it prints an "unavailable" line.
"""
from __future__ import annotations

import argparse
import atexit
import datetime
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gpu-bundle-adjustment_gb300"
GOLDEN = ROOT / "tests" / "golden"

METRIC = "LM solve s to <=1.001x oracle cost: plain FP64 vs mixed+learned PCG, 1 GB300"
TARGET_FACTOR = 1.001
MODEL = PKG / "models" / "coarse_mlp.bin"
# FP64 DMMA peak (mma.sync.m8n8k4.f64 loop) probed on a GB300 of this pool; the
# measured peaks file has no FP64 entry.


class ClockSampler:
    """SM clocks and throttle reasons during the timed region, from ONE
    long-lived `nvidia-smi -lms` process. It is started before the warm-up
    steps: each nvidia-smi start-up initialises NVML, which can stall this
    process's CUDA calls for tens of milliseconds, so no start-up may fall
    inside the timed region. Samples carry nvidia-smi's own timestamp (the
    pipe may be block-buffered); the summary keeps those inside the timed
    window, plus the nearest sample on either side when the window holds
    fewer than two."""

    QUERY = ("timestamp,clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 100

    def __init__(self, devices=("0",)):
        self.devices = ",".join(devices)  # nvidia-smi -i: physical indices or UUIDs, one line per GPU and interval
        self.samples = []  # (datetime, [sm, max, 4 reasons])
        self.window = None
        self._p = None
        self._t = None
        self._t0 = None

    def start(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", self.devices, f"--query-gpu={self.QUERY}",
                                        "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return self
        atexit.register(self.stop)
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        return self

    def _read(self):
        for line in self._p.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                continue
            self.samples.append((ts, f[1:7]))

    def begin(self):
        self._t0 = datetime.datetime.now()

    def end(self):
        self.window = (self._t0, datetime.datetime.now())

    def stop(self):
        if self._p is not None and self._p.poll() is None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._p.kill()
                self._p.wait()
        if self._t is not None:
            self._t.join(timeout=5)

    def summary(self):
        if not self.samples or self.window is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        t0, t1 = self.window
        picked = [f for ts, f in self.samples if t0 <= ts <= t1]
        n_in = len(picked)
        if n_in < 2:
            before = [(ts, f) for ts, f in self.samples if ts < t0]
            after = [(ts, f) for ts, f in self.samples if ts > t1]
            picked += [max(before, key=lambda x: x[0])[1]] if before else []
            picked += [min(after, key=lambda x: x[0])[1]] if after else []
        sm = [float(s[0]) for s in picked if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in picked if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in picked for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples_in_window": n_in, "samples_used": len(picked)}


def smi_devices(world: int, count: int):
    """nvidia-smi identifiers of the GPUs ranks 0..world-1 use on this node
    (rank r on visible device r mod count)."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    ids = [v.strip() for v in vis.split(",")] if vis else [str(i) for i in range(max(count, 1))]
    return [ids[r % len(ids)] for r in range(max(world, 1))]


def _dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The largest value over all ranks (the contract's max-over-ranks timing);
    the process group must be initialised when world > 1."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def reference_entry(workload: int, seed: int):
    """The FP64 reference solve of a workload, or None. Workloads 1-4: the
    reference's own LM driver (tests/golden/reference_runs.json); workload 5:
    the plain all-FP64 form run to convergence on a GB300
    (tests/golden/workload_reference.json), the CPU oracle being unable to
    factor its 45,000^2 system."""
    runs = GOLDEN / "reference_runs.json"
    if runs.exists():
        for e in json.loads(runs.read_text()).values():
            if e.get("workload") == workload and e.get("seed") == seed:
                return {"final_cost": e["reference"]["final_cost"], "source": "reference LM driver (src/lm.cu)"}
    f = GOLDEN / "workload_reference.json"
    if f.exists():
        e = json.loads(f.read_text()).get(f"{workload}:{seed}")
        if e is not None:
            return {"final_cost": e["final_cost"], "source": "plain FP64 form converged on a GB300"}
    return None


# ----------------------------------------------------------------- rooflines

def algorithmic_bytes(unit: str, C: int, P: int, E: int) -> float:
    """Bytes one unit of work must move (each array once), by the hot-path table's
    per-unit figures; E, P, C are the actual counts.
      matvec  one implicit FP32 Schur matvec (point pass + camera pass):
              E (108 + 4) + P (36 + 12): W_e = Jc^T Jp as 27 FP32 and a camera
              index per observation, V'^-1 (9 FP32) and the point's partial (3 FP32)
              per point; x and y (9C) stay in L2
      edge    one normal-equation accumulation with FP32 Jacobians (point pass +
              camera pass): E 132 + P 96 + C 576: indices and pixels 24 and the FP32
              W 108 per observation, the point 24 and V, bp 72 per point, U and bc
              per camera
      cost    one trial cost: E 24 + P 24 + C 72"""
    if unit == "matvec":
        return E * 112.0 + P * 48.0
    if unit == "edge":
        return E * 132.0 + P * 96.0 + C * 576.0
    if unit == "cost":
        return E * 24.0 + P * 24.0 + C * 72.0
    raise KeyError(unit)


def design_bytes(unit: str, C: int, P: int, E: int, windowed: bool = False) -> float:
    """Bytes this implementation's kernels move per unit (its own layout)."""
    if unit == "matvec" and windowed:
        # per window: point pass Jc32 72 + Jp32 24 + s_cam, s_pt 8 + u 8 (written) per slot, V'^-1 24 +
        # CSR 4 per point, x 36 per camera; camera pass: window slot index 4 per slot from HBM, the
        # window's Jc32 and u again from L2; partials 72 B per camera segment (~ per camera and window)
        return E * 116.0 + P * 28.0 + C * 36.0
    if unit == "matvec":
        # point pass: Jc32 72 + Jp32 24 + s_cam, s_pt, cam_pos 12 + u 8 per slot, V'^-1 24 + CSR 4 per
        # point, x 36 per camera; camera pass: camera record 80 + u 8 per slot
        return E * (116.0 + 88.0) + P * 28.0 + C * 36.0
    if unit == "edge":
        # point pass: indices + r 20 in, Jc32 + Jp32 96 + camera record 80 out per slot, point 24 in and
        # V / bp 72 out per point, camera record 112 per camera; camera pass: record 80 per slot
        return E * (196.0 + 80.0) + P * 96.0 + C * 112.0
    if unit == "cost":
        return E * 32.0 + P * 24.0 + C * 128.0
    raise KeyError(unit)


UNITS = {"matvec": ("schur_matvec_f32", "schur_point_pass_f32", "schur_camera_pass_f32"),
         "edge": ("point_pass_f32", "camera_pass_f32"),
         "cost": ("cost_ff",)}

# DRAM bytes (read + write) per launch from one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum, --clock-control none) of each kernel at workload 5; copied
# here, not measured in this run (profiles/schur_matvec_onepass.md,
# profiles/mixed_kernels_workload5_ncu.md).
NCU_TRAFFIC_W5 = {"point_pass_f32": 221.5e6 + 1596.8e6, "camera_pass_f32": None,
                  "schur_matvec_f32": 861.7e6 + 11.5e6 + 368.1e6 + 9.2e6,  # schur_matvec_warp + schur_matvec_long
                  "schur_point_pass_f32": 992.6e6 + 66.4e6, "schur_camera_pass_f32": 774.4e6 + 3.8e6,
                  "cost_ff": 239.9e6 + 61.0e6}

KERNELS = ("schur_matvec_f32", "schur_point_pass_f32", "schur_camera_pass_f32", "schur_point_pass_ff",
           "schur_camera_pass_ff",
           "point_pass_f32", "camera_pass_f32", "point_pass_f64", "camera_pass_f64", "cost_f64", "cost_ff",
           "backsub", "schur_rhs_point_pass", "schur_rhs_camera_pass", "mlp_forward", "schur_assemble",
           "dense_potrf", "pcg_q_finalize", "coarse_prepare", "coarse_basis", "coarse_point_pass9", "coarse_camera_pass9", "coarse_gram",
           "coarse_apply")
# stages that contain others (their times are not additional)
NESTED = {"coarse_prepare": ["coarse_basis", "coarse_point_pass9", "coarse_camera_pass9", "coarse_gram"],
          "coarse_basis": ["mlp_forward"]}


def _breakdown(solver, steps):
    out = {}
    for name in KERNELS:
        n_k, ms_k = solver.kernel_stats(name)
        if n_k:
            out[name] = {"launches": n_k, "ms_per_step": ms_k / steps}
            if name in NESTED:
                out[name]["contains"] = NESTED[name]
    return out


def roofline_mixed(solver, breakdown, C, P, E, workload, seed):
    """The unit (matvec / edge / cost) with the most device time in the timed
    region, at its measured per-launch time. The PCG matvec is re-timed on 64
    full-work iterations on the resident problem (in the timed region, launches
    after convergence inside a launch batch return early and would flatter it)."""
    peaks, peak_src = _peaks()
    share = {u: sum(breakdown.get(k, {}).get("ms_per_step", 0.0) for k in ks) for u, ks in UNITS.items()}
    unit = max(share, key=share.get)
    if share[unit] == 0.0:
        return None
    source = "timed region (CUDA events per launch on the solver stream)"
    if unit == "matvec":
        solver.reset_params()
        solver.accumulate()
        solver.damp_invert_v(1e-3)
        solver.profile_reset()
        solver.schur_pcg(1e-3, refine_tol=1e-30, refine_max_steps=1, pcg_tol=0.0, pcg_max_iters=64)
        source = "64 full-work PCG iterations (lambda 1e-3) on the resident problem, CUDA events per launch"
    per_unit_s, launches, traffic = 0.0, None, 0.0
    names = UNITS[unit]
    windowed = unit == "matvec" and solver.kernel_stats("schur_matvec_f32")[0] > 0
    if unit == "matvec":  # the windowed product is timed as one stage; the two-pass one per pass
        names = ("schur_matvec_f32",) if windowed else names[1:]
    for k in names:
        n, ms = solver.kernel_stats(k)
        if unit == "matvec":
            n = min(n, 64)
        if not n:
            return None
        per_unit_s += ms / n / 1e3
        launches = n if launches is None else min(launches, n)
        t = NCU_TRAFFIC_W5.get(k) if workload == 5 and seed == 5 else None
        traffic = None if (t is None or traffic is None) else traffic + t
    alg = algorithmic_bytes(unit, C, P, E)
    achieved = alg / per_unit_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of these kernels at workload 5, "
                               "one capture, copied into bench.py (not measured in this run)") if traffic else None,
            "kernel": "+".join(names), "work_unit": unit, "algorithmic_bytes": alg,
            "design_bytes": design_bytes(unit, C, P, E, windowed), "launches": launches,
            "avg_unit_us": per_unit_s * 1e6, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs, copy)",
            "per_launch_source": source}


_FP64_PEAK = None


def fp64_tensor_peak_tflops():
    """FP64 tensor-core peak measured in this run: cuBLAS DGEMM (torch.matmul on
    float64, 8192^3, 2 n^3 flop), best of 3 after a warm-up, CUDA events.
    MEASURED_PEAKS.json holds no FP64 entry."""
    global _FP64_PEAK
    if _FP64_PEAK is None:
        import torch

        n = 8192
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        best = float("inf")
        for _ in range(3):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            torch.cuda.synchronize()
            best = min(best, s.elapsed_time(e) / 1e3)
        _FP64_PEAK = 2.0 * n ** 3 / best / 1e12
        del a, b
    return _FP64_PEAK


def roofline_potrf(solver, C):
    n_launch, k_ms = solver.kernel_stats("dense_potrf")
    if not n_launch:
        return None
    per_launch_s = k_ms / n_launch / 1e3
    n = 9 * C
    achieved = n ** 3 / 3.0 / per_launch_s / 1e12
    peak = fp64_tensor_peak_tflops()
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": None, "kernel": "dense_potrf",
            "launches": n_launch, "avg_launch_s": per_launch_s,
            "peak_source": "measured in this run: cuBLAS DGEMM 8192^3 (FP64 tensor cores), best of 3; "
                           "MEASURED_PEAKS.json has no FP64 entry"}


# ----------------------------------------------------------------- the GPU arm

def _opts(args, target, form, **over):
    o = dict(form=form, max_iterations=args.max_iterations, target_cost=target, stop_at_target=1 if target else 0,
             refine_tol=args.refine_tol, pcg_tol=args.pcg_tol)
    if args.pcg_max_iters is not None:
        o["pcg_max_iters"] = args.pcg_max_iters
    if form == "learned":
        o["model_path"] = str(MODEL)
    o.update(over)
    return o


def _timed_steps(torch, solver, stream, opts, warmup, steps):
    """warmup untimed solves, then `steps` timed ones; returns (ms total, per-step ms, results)."""
    results = []
    for _ in range(warmup):
        solver.reset_params()
        results.append(solver.run(**opts))
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    timed = []
    start.record(stream)
    for k in range(steps):
        solver.reset_params()
        timed.append(solver.run(**opts))
        marks[k].record(stream)
    end.record(stream)
    torch.cuda.synchronize()
    step_ms = [(marks[k - 1] if k else start).elapsed_time(marks[k]) for k in range(steps)]
    return start.elapsed_time(end), step_ms, timed


def _result_summary(r, ref):
    return {"final_cost": r.final_cost, "iterations": r.iterations, "termination": r.termination,
            "time_to_target_s": r.time_to_target_s, "pcg_iterations": r.pcg_iterations, "trials": r.trials,
            "refine_steps": r.refine_steps, "max_refine_residual": r.max_refine_residual,
            "anomalies": r.anomalies,
            "learned_choice": {0: None, 1: "learned", 2: "block-Jacobi"}[r.learned_choice],
            "judged_first_solve_pcg_iterations": {"block_jacobi": r.judge_iters[0], "learned": r.judge_iters[1]},
            "rel_err_vs_fp64_reference": (r.final_cost - ref) / ref if ref else None}


def plain_denominator(torch, gba, prob, args, target):
    """One plain all-FP64 solve (dense S, DMMA Cholesky) to the same target."""
    stream = torch.cuda.Stream()
    solver = gba.Solver(prob, "plain", stream=stream.cuda_stream)
    try:
        solver.profile(True)
        opts = _opts(args, target, "plain")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        r = solver.run(**opts)
        end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        return {"time_to_target_s": start.elapsed_time(end) / 1e3, "wall_s": wall, "final_cost": r.final_cost,
                "iterations": r.iterations, "trials": r.trials, "termination": r.termination,
                "roofline": roofline_potrf(solver, prob.num_cameras), "measured": "in this run (CUDA events)"}
    finally:
        solver.close()


def plain_band(torch, gba, args):
    """The plain FP64 form on a camera path (local covisibility: S is a band):
    the same LM solve with S stored as a band (reverse Cuthill-McKee order, band
    Cholesky) and dense, CUDA events around each solve."""
    prob = gba.synthetic_local(1200, 120000, 2, 8, 1.5, 10, seed=8)
    out = {"workload": f"camera path: {prob.num_cameras} cameras / {prob.num_points} points / "
                       f"{prob.num_observations} observations, tracks within +-10 cameras, seed 8",
           "max_iterations": 10}
    runs = {}
    for layout in ("band", "dense"):
        stream = torch.cuda.Stream()
        solver = gba.Solver(prob, "plain", stream=stream.cuda_stream)
        try:
            solver.profile(True)
            opts = dict(form="plain", max_iterations=10, schur_layout=layout)
            solver.run(**opts)  # warm-up: allocates S, plans the band
            solver.profile_reset()
            solver.reset_params()
            torch.cuda.synchronize()
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record(stream)
            r = solver.run(**opts)
            end.record(stream)
            torch.cuda.synchronize()
            n_f, f_ms = solver.kernel_stats("dense_potrf")
            runs[layout] = r
            out[layout] = {"solve_s": start.elapsed_time(end) / 1e3, "iterations": r.iterations,
                           "trials": r.trials, "final_cost": r.final_cost, "band_rows": r.schur_band_rows,
                           "factorisations": n_f, "factor_ms_each": f_ms / n_f if n_f else None}
        finally:
            solver.close()
    tb, td = runs["band"].trajectory, runs["dense"].trajectory
    out["max_rel_cost_difference"] = (max(abs(a - b) / b for a, b in zip(tb, td)) if len(tb) == len(td) else None)
    out["dense_over_band"] = out["dense"]["solve_s"] / out["band"]["solve_s"]
    return out


def cpu_pair(torch, gba, args):
    """Oracle (CPU, all host cores) vs this library (learned form, same options as
    the headline) to 1.001 x the reference cost on a smaller workload."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    w = args.cpu_pair_workload
    ref = reference_entry(w, w)
    if ref is None:
        return None
    target = ref["final_cost"] * TARGET_FACTOR
    oprob = oracle.synthetic(w, w)
    threads = os.cpu_count() or 1
    o, _, _ = oracle.solve(oprob, max_iterations=args.max_iterations, threads=threads)
    k = next((i for i, c in enumerate(o["trajectory"]) if c <= target), None)
    if k is None:
        return None
    t0 = time.perf_counter()
    o2, _, _ = oracle.solve(oprob, max_iterations=k, threads=threads)
    cpu_s = time.perf_counter() - t0
    prob = gba.synthetic(w, w)
    stream = torch.cuda.Stream()
    solver = gba.Solver(prob, "learned", stream=stream.cuda_stream)
    try:
        solver.load_model(MODEL)
        ms, _, timed = _timed_steps(torch, solver, stream, _opts(args, target, "learned"), 2, 3)
    finally:
        solver.close()
    return {"workload": f"workload{w}: {prob.num_cameras} cameras / {prob.num_points} points / "
                        f"{prob.num_observations} observations, seed {w}",
            "target_cost": target, "target_source": ref["source"],
            "cpu_oracle_s": cpu_s, "cpu_cores": threads, "cpu_iterations": k, "cpu_final_cost": o2["final_cost"],
            "gpu_learned_s": ms / 3 / 1e3, "gpu_final_cost": timed[-1].final_cost,
            "gpu_iterations": timed[-1].iterations}


def cpu_sample(prob, iterations: int) -> dict:
    """CPU restatement of the reference LM (oracle/, all host threads) on a
    bounded sample of the workload, scaled to seconds per solve:
      per LM iteration >= normal-equation accumulation over all observations
                          (measured) + dense Cholesky of the 9C x 9C reduced
                          system, measured at n_sub and scaled by (9C / n_sub)^3;
    the Schur assembly, back-substitution and rejected trials are left out, so
    the figure is a lower bound on the CPU solve time; times `iterations`
    accepted LM iterations."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import numpy as np

    import oracle

    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.accumulate(prob)
    t_acc = time.perf_counter() - t0
    n = 9 * prob.num_cameras
    n_sub = min(n, 4608)
    rng = np.random.default_rng(0)
    M = rng.standard_normal((n_sub, n_sub))
    A = np.asfortranarray(M @ M.T + n_sub * np.eye(n_sub)).ravel(order="F").copy()
    t0 = time.perf_counter()
    st = oracle.cholesky(A, n_sub, threads)
    t_chol = time.perf_counter() - t0
    scale3 = (n / n_sub) ** 3
    per_iter = t_acc + t_chol * scale3
    iters = max(1, iterations)
    return {"value": per_iter * iters, "unit": "s", "cores": threads, "kind": "port",
            "extrapolated": True,
            "sample": (f"oracle normal equations over all {prob.num_observations} observations ({t_acc:.2f} s) + "
                       f"oracle dense Cholesky at n={n_sub} ({t_chol:.2f} s) scaled by (n/{n_sub})^3 to n={n}, "
                       f"x {iters} LM iterations; Schur assembly and rejected trials excluded (a lower bound, "
                       f"not a timed solve)"),
            "status": int(st)}


def run_ours(args):
    import torch

    sys.path.insert(0, str(PKG))
    import gba_gb300 as gba

    rank, world = _dist_env()
    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", dev))

    # rank 0 samples every GPU of the run, long before the timed region (see ClockSampler)
    clocks = ClockSampler(smi_devices(world, torch.cuda.device_count())) if rank == 0 else ClockSampler(())
    if rank == 0:
        clocks.start()
    prob = gba.synthetic(args.workload, args.seed)
    C, P, E = prob.num_cameras, prob.num_points, prob.num_observations
    ref = reference_entry(args.workload, args.seed)
    ref_cost = ref["final_cost"] if ref else None
    target = ref_cost * TARGET_FACTOR if ref else 0.0
    form = args.form
    opts = _opts(args, target, form)

    stream = torch.cuda.Stream()
    solver = gba.Solver(prob, form, stream=stream.cuda_stream)
    if form == "learned":
        solver.load_model(MODEL)

    # ---- headline: device-resident steps
    for _ in range(args.warmup):
        solver.reset_params()
        solver.run(**opts)
    solver.profile(True)
    solver.profile_reset()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = gba.launch_count()
    clocks.begin()
    ms_total, step_ms, timed = _timed_steps(torch, solver, stream, opts, 0, args.steps)
    clocks.end()
    launches = gba.launch_count() - l0
    ms_per_step = max_over_ranks(ms_total, world) / args.steps
    if world > 1:
        torch.distributed.barrier()
    breakdown = _breakdown(solver, args.steps)
    if form == "plain":
        roofline = roofline_potrf(solver, C)
    else:
        roofline = roofline_mixed(solver, breakdown, C, P, E, args.workload, args.seed)
    solver.profile(False)
    final = timed[-1]

    # ---- inexact Newton variant of the same form
    inexact = None
    if form != "plain" and not args.no_inexact:
        o2 = _opts(args, target, form, refine_tol=0.1, pcg_tol=0.1)
        k2 = min(args.steps, 10)
        ms2, _, t2 = _timed_steps(torch, solver, stream, o2, 2, k2)
        inexact = {"value": ms2 / k2 / 1e3, "unit": "s", "steps": k2, "refine_tol": 0.1, "pcg_tol": 0.1,
                   "note": "inexact Gauss-Newton steps: each Schur system solved to a relative residual of 0.1 "
                           "(no refinement); cost and accept / reject at FP64 accuracy",
                   "result": _result_summary(t2[-1], ref_cost)}
    solver.close()
    clocks.stop()

    # ---- e2e: gba_solve_bal on pinned host buffers, H2D + setup + solve + D2H per step
    pinned = [torch.from_numpy(a.copy()).pin_memory() for a in prob.arrays()]
    init_cams, init_pts = pinned[0].clone(), pinned[1].clone()
    h2d = sum(t.numel() * t.element_size() for t in pinned)
    d2h = pinned[0].numel() * 8 + pinned[1].numel() * 8
    e2e_times, e2e_setup = [], []
    for i in range(args.warmup + args.steps):
        pinned[0].copy_(init_cams)
        pinned[1].copy_(init_pts)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = gba.solve_raw(C, P, E, *(t.data_ptr() for t in pinned), **opts)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
            e2e_setup.append(r.phases["setup"])
    e2e_s = sum(e2e_times) / len(e2e_times)
    setup_s = sum(e2e_setup) / len(e2e_setup)

    line = {
        "metric": METRIC,
        "value": ms_per_step / 1e3,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "step_ms": [round(x, 3) for x in step_ms],
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if form == "plain" else "f32+f64",
        "data": "synthetic (seeded BAL-shaped generator; the BAL datasets are not available offline)",
        "config": {
            "workload": f"workload{args.workload}: {C} cameras / {P} points / {E} observations, seed {args.seed}",
            "form": form,
            "refine_tol": opts["refine_tol"],
            "pcg_tol": opts["pcg_tol"],
            "target_cost": target or None,
            "fp64_reference_cost": ref_cost,
            "fp64_reference_source": ref["source"] if ref else None,
            "max_iterations": args.max_iterations,
            "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas x{world}",
        },
        "result": _result_summary(final, ref_cost),
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "setup_s": setup_s, "note": "setup = device allocation, H2D of the problem, sort by point, "
                                            "camera-major view, chunking; the rest is the LM solve and the D2H"},
        "gpu_launches": launches,
        "roofline": roofline,
        "kernel_breakdown": breakdown,
        "clocks": clocks.summary(),
        "inexact_newton": inexact,
    }
    if rank == 0 and world == 1 and form != "plain" and not args.no_plain:
        line["plain_fp64_form"] = plain_denominator(torch, gba, prob, args, target)
        pl = line["plain_fp64_form"]["time_to_target_s"]
        line["plain_over_chosen"] = pl / line["value"] if pl else None
    if rank == 0 and world == 1 and not args.no_band:
        line["plain_band"] = plain_band(torch, gba, args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(prob, final.iterations)
        if args.cpu_pair_workload:
            line["cpu_pair"] = cpu_pair(torch, gba, args)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------- the CPU arm

def run_reference(args):
    """The oracle's LM solve on the host cores, nothing of this library loaded.
    Workloads whose dense reduced camera system does not fit a few minutes of
    CPU time (more than --reference-max-cameras cameras) are timed on a bounded
    sample per step (cpu_sample: the normal equations over all observations
    plus the dense Cholesky at n = 4,608, scaled to the full system; a lower
    bound on the solve, as its sample string says)."""
    rank, world = _dist_env()
    if rank != 0:
        return
    C = {1: 16, 2: 257, 3: 1000, 4: 1000, 5: 5000}.get(args.workload)
    if C is not None and C > args.reference_max_cameras:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle

        prob = oracle.synthetic(args.workload, args.seed)
        ref = reference_entry(args.workload, args.seed)
        target = ref["final_cost"] * TARGET_FACTOR if ref else None
        traj = None
        f = GOLDEN / "workload_reference.json"
        if f.exists():
            traj = json.loads(f.read_text()).get(f"{args.workload}:{args.seed}", {}).get("trajectory")
        iters = next((i for i, c in enumerate(traj) if c <= target), None) if (traj and target) else None
        iters = iters or args.max_iterations
        samples = []
        for i in range(args.warmup + args.steps):
            smp = cpu_sample(prob, iters)
            if i >= args.warmup:
                samples.append(smp)
        v = sum(x["value"] for x in samples) / len(samples)
        line = {
            "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded BAL-shaped generator)",
            "config": {"workload": f"workload{args.workload}: {prob.num_cameras} cameras / {prob.num_points} "
                                   f"points / {prob.num_observations} observations, seed {args.seed}",
                       "form": "plain (CPU oracle)", "target_cost": target, "iterations_to_target": iters},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "s", "cores": samples[-1]["cores"], "kind": "port",
                             "extrapolated": True, "sample": "per step: " + samples[-1]["sample"]},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    if C is None:
        print(json.dumps({"impl": "reference", "unavailable": f"unknown workload {args.workload}"}))
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    prob = oracle.synthetic(args.workload, args.seed)
    ref = reference_entry(args.workload, args.seed)
    target = ref["final_cost"] * TARGET_FACTOR if ref else None
    threads = os.cpu_count() or 1
    o, _, _ = oracle.solve(prob, max_iterations=args.max_iterations, threads=threads)
    k = (next((i for i, c in enumerate(o["trajectory"]) if c <= target), None) if target else None)
    iters = k if k is not None else args.max_iterations
    vals = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        oracle.solve(prob, max_iterations=iters, threads=threads)
        if i >= args.warmup:
            vals.append(time.perf_counter() - t0)
    v = sum(vals) / len(vals)
    line = {
        "metric": METRIC, "value": v, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded BAL-shaped generator)",
        "config": {"workload": f"workload{args.workload}: {prob.num_cameras} cameras / {prob.num_points} points / "
                               f"{prob.num_observations} observations, seed {args.seed}",
                   "form": "plain (CPU oracle)", "target_cost": target, "iterations_to_target": k},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port",
                         "sample": f"whole oracle LM solves to the target ({iters} iterations) per step"},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", type=int, default=5)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--form", default="learned", choices=["plain", "mixed", "learned"])
    ap.add_argument("--max-iterations", type=int, default=50)
    ap.add_argument("--pcg-tol", type=float, default=1e-4, help="inner PCG relative tolerance")
    ap.add_argument("--refine-tol", type=float, default=1e-8, help="relative residual target of each Schur step")
    ap.add_argument("--pcg-max-iters", type=int, default=None)
    ap.add_argument("--no-inexact", action="store_true", help="skip the inexact-Newton extra measurement")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 solve to the target")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-band", action="store_true", help="skip the plain form's band-vs-dense camera-path solve")
    ap.add_argument("--cpu-pair-workload", type=int, default=2)
    ap.add_argument("--reference-max-cameras", type=int, default=300,
                    help="largest workload (cameras) the CPU arm solves whole; above it, a bounded sample per step")
    args = ap.parse_args()
    if args.seed is None:
        args.seed = args.workload
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
