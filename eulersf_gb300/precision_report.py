"""Mixed precision against the FP64 path on the same scene: both integrators
start from the same state and step side by side; per step it reports each
path's device time and solver iterations, the mixed path's relative
residuals, and the L-inf differences of velocity, pressure (lambda1) and
solid displacement between the two trajectories, relative to the FP64
field's max-norm.

    python -m eulersf_gb300.precision_report [--size 256] [--steps 6] [--seed 7] [--x64]
    python -m eulersf_gb300.precision_report --fp64-only --size 128 --steps 50 --seed 0

--x64 steps a third integrator at ESF_MIXED_X64 (one FP32 pressure run per
solve with a double-float correction and direction) beside the two.

Prints one JSON line per step and a summary line.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import abi, make_scene
from .scene import SceneDesc, SolidDesc


def _linf(a, b):
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    s = float(np.abs(b).max()) if b.size else 0.0
    d = float(np.abs(a - b).max()) if b.size else 0.0
    return d / s if s > 0 else d


def run_fp64(size=128, steps=50, seed=0, mass_sample_dh=None, out=print):
    """The plain FP64 path alone (the benchmark's plain-method configurations):
    per step its device time, wall time and solver iterations, and a summary
    of steps/s, cells/s and pressure iterations/s."""
    import time
    desc = SceneDesc(N=size, noise_seed=seed, mass_sample_dh=mass_sample_dh or (1.0 / size) / 4,
                     solids=[SolidDesc(center=(0.5, 0.65, 0.5), radius=0.15, density=1100.0,
                                       E=2e5, nu=0.45)])
    A = make_scene(desc, precision=abi.ESF_FP64)
    rows = []
    for k in range(steps):
        t0 = time.perf_counter()
        r = A.stepImplicit()
        rows.append({"step": k, "device_ms": r["device_ms"], "wall_ms": (time.perf_counter() - t0) * 1e3,
                     "iterations": r["iterations"], "rel_residual": max(r["rel_residual"])})
        out(json.dumps(rows[-1]))
    A.close()
    t = sum(r["device_ms"] for r in rows) * 1e-3
    tw = sum(r["wall_ms"] for r in rows) * 1e-3
    piters = sum(r["iterations"][1] for r in rows)
    summary = {"summary": True, "precision": "fp64", "size": size, "steps": steps, "seed": seed,
               "mass_sample_dh": desc.mass_sample_dh, "steps_per_s": steps / t, "wall_steps_per_s": steps / tw,
               "cells_per_s": size ** 3 * steps / t, "pressure_iters_per_s": piters / t,
               "pressure_iters_per_step": piters / steps,
               "max_rel_residual": max(r["rel_residual"] for r in rows)}
    out(json.dumps(summary))
    return rows, summary


def run(size=256, steps=6, seed=7, out=print, x64=False):
    desc = SceneDesc(N=size, noise_seed=seed,
                     solids=[SolidDesc(center=(0.5, 0.65, 0.5), radius=0.15, density=1100.0,
                                       E=2e5, nu=0.45)])
    A = make_scene(desc, precision=abi.ESF_FP64)
    B = make_scene(desc, precision=abi.ESF_MIXED)
    X = make_scene(desc, precision=abi.ESF_MIXED_X64) if x64 else None
    ta = tb = tx = 0.0
    rows = []
    for k in range(steps):
        ra, rb = A.stepImplicit(), B.stepImplicit()
        ta += ra["device_ms"]
        tb += rb["device_ms"]
        row = {"step": k, "fp64_ms": ra["device_ms"], "mixed_ms": rb["device_ms"],
               "fp64_iterations": ra["iterations"], "mixed_iterations": rb["iterations"],
               "mixed_fp64_finish_iterations": rb["fp64_iterations"],
               "mixed_refinements": rb["refinements"], "fp64_rel_residual": ra["rel_residual"],
               "mixed_rel_residual": rb["rel_residual"], "mixed_converged": rb["converged"],
               "linf_velocity": _linf(B.get("velocity"), A.get("velocity")),
               "linf_pressure": _linf(B.get("lambda1"), A.get("lambda1")),
               "linf_solid_displacement": _linf(B.get("solid.u"), A.get("solid.u")),
               "dt": [ra["dt"], rb["dt"]]}
        if X is not None:
            rx = X.stepImplicit()
            tx += rx["device_ms"]
            row.update({"x64_ms": rx["device_ms"], "x64_iterations": rx["iterations"],
                        "x64_checks": rx["refinements"][1], "x64_rel_residual": rx["rel_residual"],
                        "x64_converged": rx["converged"],
                        "x64_linf_velocity": _linf(X.get("velocity"), A.get("velocity")),
                        "x64_linf_pressure": _linf(X.get("lambda1"), A.get("lambda1"))})
        rows.append(row)
        out(json.dumps(row))
    summary = {"summary": True, "size": size, "steps": steps, "seed": seed,
               "fp64_steps_per_s": steps / (ta * 1e-3), "mixed_steps_per_s": steps / (tb * 1e-3),
               "speedup": ta / tb if tb > 0 else None,
               "max_linf_velocity": max(r["linf_velocity"] for r in rows),
               "max_linf_pressure": max(r["linf_pressure"] for r in rows),
               "max_mixed_rel_residual": max(max(r["mixed_rel_residual"]) for r in rows)}
    if X is not None:
        summary.update({"x64_steps_per_s": steps / (tx * 1e-3), "x64_speedup": ta / tx if tx > 0 else None,
                        "x64_max_linf_velocity": max(r["x64_linf_velocity"] for r in rows),
                        "x64_max_linf_pressure": max(r["x64_linf_pressure"] for r in rows),
                        "x64_max_rel_residual": max(max(r["x64_rel_residual"]) for r in rows)})
        X.close()
    out(json.dumps(summary))
    A.close()
    B.close()
    return rows, summary


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--fp64-only", action="store_true", help="the plain FP64 path alone")
    ap.add_argument("--mass-sample-dh", type=float, default=None)
    ap.add_argument("--x64", action="store_true", help="also step an ESF_MIXED_X64 integrator")
    a = ap.parse_args(argv)
    if a.fp64_only:
        run_fp64(a.size, a.steps, a.seed, a.mass_sample_dh)
    else:
        run(a.size, a.steps, a.seed, x64=a.x64)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
