"""The large two-sphere scene: one 384^3 scene, fluid height 0.3, two elastic
spheres of radius 0.12 (density 1100, E 3e5, nu 0.45) at (0.35, 0.7, 0.5)
and (0.65, 0.8, 0.5), each with its rest SDF for solid-solid contact,
stepped in mixed precision (FP32 inner solves inside FP64 refinement to
1e-8).

Per step it prints the device time, the solver iterations, the mixed path's
relative residuals, whether the broad phase flagged a contact (CFL 0.6) and
how many particles took a solid-solid impulse; the summary gives steps/s,
cells/s and pressure iterations/s, and the pressure iteration kernel's
device time per launch as a fraction of the measured HBM copy bandwidth
(the roofline of the step: 64-88% of it is the pressure solve).

    python -m eulersf_gb300.two_sphere_bench [--size 384] [--steps 10] [--seed 7]
    python -m eulersf_gb300.two_sphere_bench --collide      # the same balls, touching and approaching
    python -m eulersf_gb300.two_sphere_bench --precision mixed-x64   # ESF_MIXED_X64 pressure solves

--collide places the two balls side by side at (0.38, 0.7, 0.5) and
(0.62, 0.7, 0.5), 0.24 apart centre to centre, moving towards each other at
0.5 m/s, so that solid-solid contact acts from the first step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

from . import abi, load, make_scene
from .scene import SceneDesc, SolidDesc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def scene(size: int = 384, seed: int = 7, collide: bool = False) -> SceneDesc:
    if collide:
        balls = [SolidDesc(center=c, radius=0.12, density=1100.0, E=3e5, nu=0.45, velocity=v)
                 for c, v in (((0.38, 0.7, 0.5), (0.5, 0.0, 0.0)), ((0.62, 0.7, 0.5), (-0.5, 0.0, 0.0)))]
    else:
        balls = [SolidDesc(center=c, radius=0.12, density=1100.0, E=3e5, nu=0.45)
                 for c in ((0.35, 0.7, 0.5), (0.65, 0.8, 0.5))]
    return SceneDesc(N=size, noise_seed=seed, fluid_height=0.3, solids=balls)


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run(size=384, steps=10, seed=7, out=print, collide=False, precision="mixed"):
    desc = scene(size, seed, collide)
    prec = abi.ESF_MIXED_X64 if precision == "mixed-x64" else abi.ESF_MIXED
    t0 = time.perf_counter()
    I = make_scene(desc, precision=prec)
    setup_s = time.perf_counter() - t0
    rows = []
    for k in range(steps):
        t1 = time.perf_counter()
        r = I.stepImplicit()
        rows.append({"step": k, "device_ms": r["device_ms"], "wall_ms": (time.perf_counter() - t1) * 1e3,
                     "iterations": r["iterations"], "refinements": r["refinements"],
                     "rel_residual": r["rel_residual"], "converged": r["converged"],
                     "prone_to_contact": r["prone_to_contact"], "solid_contacts": r["solid_contacts"],
                     "fp64_stress_cells": r["fp64_stress_cells"], "valid_cells": r["valid_cells"],
                     "dt": r["dt"], "phase_ms": r["phase_ms"]})
        out(json.dumps(rows[-1]))
    # the one-pass FP32 pressure iteration on this scene's pressure problem
    upd, axpy = C.c_double(), C.c_double()
    st = load().esf_time_pressure_kernels(I._h, 20, C.byref(upd), C.byref(axpy))
    I.close()
    R = size ** 3
    t = sum(r["device_ms"] for r in rows) * 1e-3
    piters = sum(r["iterations"][1] for r in rows)
    peak, kind = hbm_peak()
    words = 17  # per row of a whole iteration but its residual check, 4-byte words
    moved = 16 if prec == abi.ESF_MIXED_X64 else 12  # the words the one-pass kernel moves
    achieved = words * 4 * R / (upd.value * 1e-3) / 1e9 if st == 0 and upd.value > 0 else None
    summary = {"summary": True, "scene": "two spheres, radius 0.12, fluid height 0.3"
               + (", touching and approaching" if collide else ""), "size": size,
               "steps": steps, "seed": seed, "precision": precision, "setup_s": setup_s,
               "steps_per_s": steps / t, "cells_per_s": R * steps / t,
               "pressure_iters_per_s": piters / t, "pressure_iters_per_step": piters / steps,
               "max_rel_residual": max(max(r["rel_residual"]) for r in rows),
               "all_converged": all(all(r["converged"]) for r in rows),
               "steps_prone_to_contact": sum(r["prone_to_contact"] for r in rows),
               "solid_contacts": sum(r["solid_contacts"] for r in rows),
               "pressure_kernel_us": upd.value * 1e3 if st == 0 else None,
               "pressure_kernel_gbs": achieved, "hbm_peak_gbs": peak, "peak_kind": kind,
               "hbm_frac": achieved / peak if achieved else None,
               "moved_words": moved,
               "frac_of_moved": (moved * 4 * R / (upd.value * 1e-3) / 1e9 / peak) if achieved else None,
               "note": "hbm_frac: the one-pass pressure iteration's 17 four-byte words per row "
                       "over its CUDA-event time per launch, against the measured copy bandwidth"}
    out(json.dumps(summary))
    return rows, summary


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=384)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--collide", action="store_true", help="balls touching and approaching")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed-x64"])
    a = ap.parse_args(argv)
    run(a.size, a.steps, a.seed, collide=a.collide, precision=a.precision)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
