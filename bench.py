"""Benchmark of the coupled solid-fluid step on GB300.

Workload (one "step" = one stepImplicit of the scene): the rubber-ball scene
at 256^3 cells (257^3 nodes, dx = 1/256), sphere r = 0.15 at (0.5, 0.65, 0.5),
density 1100, E = 2e5, nu = 0.45, fluid density 1000, gravity 9.8,
dt = 1/240, all solves to 1e-8 relative residual, seeded fluid noise
(seed 7), mixed precision (FP32 inner PCR in FP64 refinement). Synthetic
input: the scene generator of eulersf_gb300/scene.py. Every working array
the pressure iterations stream (>= 67 MB each, ~4 GB in all) is larger than
the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one scene per GPU): the step does not
shard. Prints one JSON line (rank 0).

Beside the mixed-precision headline, a single-GPU run also steps the plain
FP64 GPU path over the first steps of the same scene (--fp64-steps, default
3: steps 1..3, after an untimed step 0 that both paths take) and reports
the ratio of the two paths' steps/s on those steps, each path's pressure
iterations, and the L-inf differences of velocity and pressure between them
after each compared step; and it re-checks the final mixed pressure solve's
relative residual with the CPU oracle's operator (outside the timed region).
It then runs the same steps once more with precision ESF_MIXED_X64 (the
pressure solve's iterate and direction in FP64, one Krylov run per solve:
`mixed_x64`, --no-x64 to skip), outside the timed region of `value`.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "coupled steps/s and CG iters/s at 256^3 (mixed vs FP64 GPU)"
UNIT = "steps/s"
# Pressure PCR iterations per step of the reference's FP64 algorithm on this
# workload, steps 0-29, counted by the FP64 GPU path (its counts match the
# reference's build to within one 5-iteration check interval at 64^3 over 20
# steps): profiles/mixed_vs_fp64_256.md. Later steps use the mean of steps
# 27-29. A single-GPU run re-counts its first steps live (fp64_gpu) and
# reports whether they agree with this table.
FP64_PRESSURE_ITERS_256 = [19060, 14655, 9545, 8925, 6770, 5385, 5740, 5360, 5795, 6785,
                           6615, 5390, 6790, 7325, 5665, 6930, 8310, 6650, 12150, 14465,
                           14565, 11800, 10665, 20430, 13165, 10400, 9745, 10470, 10325, 14700]


def fp64_iters(step):
    t = FP64_PRESSURE_ITERS_256
    return t[step] if step < len(t) else sum(t[-3:]) / 3.0


def fp64_iters_window(warmup, steps):
    """FP64 pressure iterations per step over the timed steps warmup .. warmup+steps-1."""
    return sum(fp64_iters(k) for k in range(warmup, warmup + steps)) / steps


def workload(N=256, seed=7):
    from eulersf_gb300.scene import SceneDesc, SolidDesc
    return SceneDesc(N=N, noise_seed=seed,
                     solids=[SolidDesc(center=(0.5, 0.65, 0.5), radius=0.15, density=1100.0,
                                       E=2e5, nu=0.45)])


def config_dict(desc, precision, n_gpus):
    return {"workload": f"rubber ball {desc.N}^3 cells ({desc.res}^3 nodes), r=0.15, E=2e5, nu=0.45, "
                        f"fluid 1000 / solid 1100, dt=1/240, tol 1e-8, seed {desc.noise_seed}",
            "grid_cells": desc.N ** 3, "precision": precision, "parallelism": f"replicas x{n_gpus}",
            "l2": "inputs larger than L2 (no flush)"}


def _linf(a, b):
    """max |a - b| / max |b| (b the FP64 field)."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    s = float(np.abs(b).max()) if b.size else 0.0
    d = float(np.abs(a - b).max()) if b.size else 0.0
    return d / s if s > 0 else d


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def start(self):
        cmd = ["nvidia-smi", "-i", str(self.gpu),
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
               "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
               "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
               "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def dist_setup(n_gpus):
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("ESF_BENCH_GLOO") is None else "gloo")
        pg = dist
    return rank, world, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def _reduce_device(pg):
    # NCCL reduces device tensors; gloo (ESF_BENCH_GLOO, the CPU tests) host ones
    return "cuda" if pg.get_backend() == "nccl" else "cpu"


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device(pg))
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device(pg))
    pg.all_reduce(t)
    return float(t.item())


# --------------------------------------------------------- CPU baseline
def cpu_pressure_sample(desc, iters, threads=None):
    """Time `iters` FP64 pressure-PCR iterations at the workload's size with
    the CPU oracle (the reference's algorithm restated in C, OpenMP on the
    operator and the elementwise updates)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    from eulersf_gb300.scene import pressure_problem
    minv, diag, b = pressure_problem(desc)
    g = oracle.grid(desc.res, desc.dh)
    oracle.pressure_apply(g, minv, b)  # load + first touch
    t0 = time.perf_counter()
    _, it, _, _ = oracle.pressure_solve(g, minv, diag, b, np.zeros_like(b), 1e-30, iters)
    return it, time.perf_counter() - t0


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_arm(args):
    """--impl reference: the reference algorithm on the host cores (the
    oracle port; the reference's own binaries are built for this machine
    only), same workload, metric and unit."""
    rank, world, pg = dist_setup(args.gpus)
    if rank != 0:
        return 0
    desc = workload(args.size)
    threads = cpu_threads()
    per_step = []
    sample_iters = max(2, args.cpu_iters)
    for _ in range(args.warmup):
        cpu_pressure_sample(desc, 1, threads)
    for k in range(args.warmup, args.warmup + args.steps):
        it, t = cpu_pressure_sample(desc, sample_iters, threads)
        per_step.append(t / max(it, 1) * fp64_iters(k))
    t_step = statistics.mean(per_step)
    value = 1.0 / t_step
    sample = (f"{sample_iters} FP64 pressure-PCR iterations at {desc.N}^3 per timed step "
              f"(oracle port, {threads} threads); each step's time = time per iteration x the "
              f"reference algorithm's pressure iterations of that step (steps {args.warmup}.."
              f"{args.warmup + args.steps - 1}: {fp64_iters_window(args.warmup, args.steps):.0f} per step); "
              f"the non-solver part of the step (<2% at this tolerance) is not counted")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_dict(desc, "fp64 (reference algorithm)", args.gpus),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "extrapolated": True, "sampled_iterations_per_step": sample_iters,
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------- our arm
def ours(args):
    import torch
    rank, world, pg = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(local)
    import eulersf_gb300 as E
    from eulersf_gb300 import abi
    lib = E.load()
    prec = abi.ESF_MIXED if args.precision == "mixed" else abi.ESF_FP64
    desc = workload(args.size)
    stream = torch.cuda.current_stream()
    I = E.make_scene(desc, precision=prec, stream=stream.cuda_stream)
    # the FP64 comparison covers steps 1..F, which the warm-up takes (step 0
    # carries the first step's one-time set-up on both paths)
    compare = (world == 1 and prec == abi.ESF_MIXED and not args.no_fp64)
    F = max(0, min(args.fp64_steps, args.warmup - 1)) if compare else 0
    warm_reports, snaps = [], {}
    for k in range(args.warmup):
        warm_reports.append(I.stepImplicit())
        if 1 <= k <= F:
            snaps[k] = (I.get("velocity"), I.get("lambda1"))
    # ---- timed region. Every step goes through the public C ABI: the step's
    # input field (intensity, the smoke source) is copied in from pinned host
    # memory, esf_step runs, and its result (the velocity field) is copied
    # out. `value` is the device time of the steps alone (CUDA events around
    # esf_step on the scene stream, inputs resident); `e2e` is the wall time
    # of the whole loop including both copies.
    res = desc.res
    h_in = torch.from_numpy(I.get("intensity")).pin_memory()
    h_out = torch.empty(res ** 3 * 3, dtype=torch.float64).pin_memory()
    fid_in, fid_out = abi.FIELDS["intensity"][0], abi.FIELDS["velocity"][0]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    reports = []
    rep = abi.StepReport()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(pg)
    torch.cuda.synchronize()
    l0 = lib.esf_kernel_launches()
    torch.cuda.nvtx.range_push("timed")
    t0 = time.perf_counter()
    for k in range(args.steps):
        st_in = lib.esf_set_field(I._h, fid_in, 0, C.c_void_p(h_in.data_ptr()), h_in.numel() * 8)
        ev[k][0].record(stream)
        st = lib.esf_step(I._h, C.byref(rep))
        ev[k][1].record(stream)
        st_out = lib.esf_get_field(I._h, fid_out, 0, C.c_void_p(h_out.data_ptr()), h_out.numel() * 8)
        if st_in or st_out or st not in (0, 6):  # 6: ESF_ERR_NUMERIC, carried in the report
            raise RuntimeError(f"step {k}: status {st_in}/{st}/{st_out}: {E.last_error()}")
        reports.append(rep.as_dict())
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    barrier(pg)
    launches = lib.esf_kernel_launches() - l0
    clk = clocks.stop()
    t = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    t_max = max_over_ranks(pg, t)
    te = max_over_ranks(pg, t_wall)
    steps_all = sum_over_ranks(pg, args.steps)
    value = steps_all / t_max
    piters = sum(r["iterations"][1] for r in reports)
    cg_rate = sum_over_ranks(pg, piters) / t_max
    e2e = {"value": steps_all / te, "unit": UNIT,
           "h2d_bytes_per_step": int(h_in.numel() * 8), "d2h_bytes_per_step": int(h_out.numel() * 8),
           "what": "the timed steps themselves, each with the intensity field copied in and the "
                   "velocity field copied out through pinned host buffers (esf_set_field, esf_step, "
                   "esf_get_field)"}
    # ---- independent check of the last mixed pressure solve: its relative
    # residual with the CPU oracle's operator (rank 0, N=1; outside the timing)
    final_check = None
    if rank == 0 and world == 1 and not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        tr = time.perf_counter()
        res = oracle.pressure_residual(I)
        final_check = {"relative_residual": res, "step": args.warmup + args.steps - 1,
                       "gpu_reported": max(reports[-1]["rel_residual"]),
                       "seconds": time.perf_counter() - tr,
                       "what": "||J M^-1 J^T lambda1 - b1|| / ||b1|| of the last timed step's pressure "
                               "solve, evaluated by the oracle on the host"}
    # ---- dominant kernel of the pressure PCR: the one-pass FP32 iteration
    # (mixed, rows a multiple of 4 floats) or the update + stencil + dot kernel
    upd, axpy = C.c_double(), C.c_double()
    stt = lib.esf_time_pressure_kernels(I._h, 20, C.byref(upd), C.byref(axpy))
    R = desc.N ** 3
    w = 4 if prec == abi.ESF_MIXED else 8
    peak, peak_kind = read_peaks()
    one_pass = stt == 0 and w == 4 and axpy.value == 0.0
    # algorithmic words per row of the 17.6-word per-iteration model: a whole
    # iteration without the residual check (P1 + P2 + P3) for the one-pass
    # kernel, P2 + P3 for the update kernel; and the words each must move
    words, moved = (17, 12) if one_pass else (10, 8)
    algo = words * w * R
    achieved = algo / (upd.value * 1e-3) / 1e9 if stt == 0 and upd.value > 0 else None
    moved_gbs = moved * w * R / (upd.value * 1e-3) / 1e9 if achieved else None
    traffic = None
    tp = os.path.join(ROOT, "profiles", "pressure_update_traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        traffic = tj.get(f"{'fp32' if w == 4 else 'fp64'}_{desc.N}{'_one_pass' if one_pass else ''}")
    if one_pass:
        kname = "pcr_iteration_fused"
    else:
        kname = ("pressure_update_tma" if (w == 4 and desc.N % 4 == 0) else
                 f"pressure_stencil<{'float' if w == 4 else 'double'}, update>")
    dram_gbs = traffic / (upd.value * 1e-3) / 1e9 if (traffic and achieved) else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                "peak_kind": peak_kind, "kernel": kname,
                "kernel_ms": upd.value, "axpy_kernel_ms": axpy.value,
                "algorithmic_bytes_per_launch": algo,
                "words_per_row": {"algorithmic": words, "moved": moved},
                "moved_bytes_per_launch": moved * w * R,
                "frac_of_moved": (moved_gbs / peak) if moved_gbs else None,
                "dram_achieved_gbs": dram_gbs,
                "dram_frac": (dram_gbs / peak) if dram_gbs else None,
                "note": "achieved/frac count the per-iteration model's words (a whole iteration but "
                        "its residual check: 17 words a row); the one-pass kernel folds the Jacobi "
                        "scaling into its vectors and moves 12 (frac_of_moved); dram_* divide the "
                        "ncu-measured DRAM bytes of one launch (traffic, with L2 compression) by "
                        "the same duration"}
    # ---- the plain FP64 GPU path on the same scene, steps 1..F
    fp64 = None
    fsnaps = {}
    if F > 0:
        I.close()  # the mixed scene's memory is not needed any more
        I = None
        D = E.make_scene(desc, precision=abi.ESF_FP64, stream=stream.cuda_stream)
        rows = []
        for k in range(F + 1):
            r = D.stepImplicit()
            if k == 0:
                continue
            fsnaps[k] = (D.get("velocity"), D.get("lambda1"), r["device_ms"])
            vm, lm = snaps[k]
            rows.append({"step": k, "fp64_ms": r["device_ms"], "mixed_ms": warm_reports[k]["device_ms"],
                         "fp64_pressure_iters": r["iterations"][1],
                         "mixed_pressure_iters": warm_reports[k]["iterations"][1],
                         "fp64_rel_residual": max(r["rel_residual"]),
                         "mixed_rel_residual": max(warm_reports[k]["rel_residual"]),
                         "l_inf_velocity": _linf(vm, D.get("velocity")),
                         "l_inf_pressure": _linf(lm, D.get("lambda1"))})
        D.close()
        t64 = sum(r["fp64_ms"] for r in rows) * 1e-3
        tmx = sum(r["mixed_ms"] for r in rows) * 1e-3
        table = [fp64_iters(r["step"]) for r in rows]
        fp64 = {"steps": [r["step"] for r in rows],
                "fp64_gpu_steps_per_s": len(rows) / t64, "mixed_steps_per_s_same_steps": len(rows) / tmx,
                "mixed_over_fp64": t64 / tmx,
                "fp64_pressure_iters_each_step": [r["fp64_pressure_iters"] for r in rows],
                "fp64_iters_match_table": [r["fp64_pressure_iters"] for r in rows] == table,
                "mixed_pressure_iters_each_step": [r["mixed_pressure_iters"] for r in rows],
                "l_inf_velocity_each_step": [r["l_inf_velocity"] for r in rows],
                "l_inf_pressure_each_step": [r["l_inf_pressure"] for r in rows],
                "rel_residual_max": {"fp64": max(r["fp64_rel_residual"] for r in rows),
                                     "mixed": max(r["mixed_rel_residual"] for r in rows)},
                "what": "both paths from the same initial state, steps 1..F (step 0 untimed on both: "
                        "first-step set-up); device time of each step (CUDA events in esf_step); "
                        "L-inf = max |mixed - fp64| / max |fp64| of the field after the step"}
    # ---- the same workload with the pressure solve's iterate and direction
    # in FP64 (ESF_MIXED_X64: one FP32 Krylov run per solve, no restarts),
    # over the same warm-up and timed steps; device time from the step reports
    x64 = None
    if compare and not args.no_x64:
        if I is not None:
            I.close()
            I = None
        X = E.make_scene(desc, precision=abi.ESF_MIXED_X64, stream=stream.cuda_stream)
        xr, lv, lp, t64s, txs = [], [], [], 0.0, 0.0
        for k in range(args.warmup + args.steps):
            r = X.stepImplicit()
            xr.append(r)
            if k in fsnaps:
                vf, lf, ms64 = fsnaps[k]
                lv.append(_linf(X.get("velocity"), vf))
                lp.append(_linf(X.get("lambda1"), lf))
                t64s += ms64 * 1e-3
                txs += r["device_ms"] * 1e-3
        timed = xr[args.warmup:]
        tx = sum(r["device_ms"] for r in timed) * 1e-3
        xu, xa = C.c_double(), C.c_double()
        stx = lib.esf_time_pressure_kernels(X._h, 20, C.byref(xu), C.byref(xa))
        X.close()
        moved_x = 16 * 4 * R
        x_gbs = moved_x / (xu.value * 1e-3) / 1e9 if stx == 0 and xu.value > 0 else None
        x64 = {"steps_per_s": args.steps / tx, "over_mixed": (args.steps / tx) / value,
               "over_fp64_same_steps": (t64s / txs) if txs > 0 else None,
               "pressure_iters_each_step": [r["iterations"][1] for r in timed],
               "pressure_iters_per_step": sum(r["iterations"][1] for r in timed) / args.steps,
               "fp64_checks_each_step": [r["refinements"][1] for r in timed],
               "rel_residual_max": max(max(r["rel_residual"]) for r in xr),
               "all_converged": all(all(r["converged"]) for r in xr),
               "l_inf_velocity_each_step": lv, "l_inf_pressure_each_step": lp,
               "kernel": "pcr_iteration_fused_x64", "kernel_ms": xu.value if stx == 0 else None,
               "moved_words_per_row": 16, "frac_of_moved": (x_gbs / peak) if x_gbs else None,
               "what": "precision ESF_MIXED_X64 on the same scene and steps: FP32 operator, residual "
                       "vectors and stencil; the pressure solve's iterate and search direction in "
                       "FP64; one Krylov run per solve to the 1e-8 FP64 residual, checked in FP64 "
                       "(no inner tolerance, no restarts). Not the configured refinement (FP32 inner "
                       "solves to 1e-4), which `value` measures. L-inf against the FP64 path after "
                       "steps 1..F; over_fp64_same_steps on those steps"}
    # ---- CPU baseline (rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = cpu_threads()
        it, tc = cpu_pressure_sample(desc, args.cpu_iters, threads)
        per_iter = tc / max(it, 1)
        t_step = per_iter * fp64_iters_window(args.warmup, args.steps)
        cpu = {"value": 1.0 / t_step, "unit": UNIT, "cores": threads, "kind": "port",
               "extrapolated": True, "sampled_iterations": it, "sample_seconds": tc, "seconds_per_iteration": per_iter,
               "fp64_iters_per_step": fp64_iters_window(args.warmup, args.steps),
               "sample": f"{it} FP64 pressure-PCR iterations at {desc.N}^3 on the oracle port "
                         f"({tc:.1f} s, {threads} threads); steps/s = 1 / (time per iteration x "
                         f"{fp64_iters_window(args.warmup, args.steps):.0f}, the reference algorithm's "
                         f"pressure iterations per step over the same steps "
                         f"{args.warmup}..{args.warmup + args.steps - 1}, counted by the FP64 GPU path); "
                         f"non-solver work not counted"}
        if final_check is not None:
            cpu["residual_check"] = final_check
    if rank == 0:
        last = reports[-1]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer" if w == 4 else "f64",
            "data": "synthetic (seeded scene generator)", "config": config_dict(desc, args.precision, world),
            "cg_iters_per_s": cg_rate, "pressure_iters_per_step": piters / args.steps,
            "pressure_iters_each_step": [r["iterations"][1] for r in reports],
            "fp64_pressure_iters_same_steps": fp64_iters_window(args.warmup, args.steps),
            "solid_iters_per_step": [r["iterations"][0] + r["iterations"][2] for r in reports],
            "refinements_last_step": last["refinements"],
            "rel_residual_max": max(max(r["rel_residual"]) for r in reports),
            "phase_ms_last_step": last["phase_ms"], "roofline": roofline, "cpu_baseline": cpu,
            "fp64_gpu": fp64,
            "mixed_over_fp64": fp64["mixed_over_fp64"] if fp64 else None,
            "fp64_gpu_steps_per_s": fp64["fp64_gpu_steps_per_s"] if fp64 else None,
            "l_inf_velocity": max(fp64["l_inf_velocity_each_step"]) if fp64 else None,
            "l_inf_pressure": max(fp64["l_inf_pressure_each_step"]) if fp64 else None,
            "mixed_x64": x64,
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if I is not None:
        I.close()
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-iters", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=3,
                    help="FP64 GPU comparison over steps 1..F (bounded by --warmup - 1)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-x64", action="store_true",
                    help="skip the ESF_MIXED_X64 run of the same steps (mixed_x64)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
