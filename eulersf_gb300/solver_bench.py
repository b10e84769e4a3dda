"""Pressure-solver throughput through the solver seam (esf_pressure_solve,
the replacement of CONJUGATE_RESIDUAL::solvePCR with getMatVecMult,
CONJUGATE_RESIDUAL.inl:109-192, COUPLED_INTEGRATOR_3D.cpp:638-660): PCR
iterations per second ("CG iters/s") on a pressure system of the rubber-ball
scene's size, device-resident inputs, timed with CUDA events on the stream
the solve runs on.

    python -m eulersf_gb300.solver_bench [--size 256] [--precision mixed|mixed-x64|fp64]
                                         [--iters 300] [--repeat 3] [--batch B [--autotune]]

The tolerance is set to 1e-30 so every solve runs exactly --iters
iterations (mixed: FP32 inner iterations summed over the refinements).
With --batch B, B independent systems of the size (different seeded
right-hand sides) are solved by one esf_pressure_solve_batch call, their
inner iterations sharing launches; the line reports the aggregate
iterations/s by wall clock around the call, the marginal rate of a 4x
longer call (per-call set-up left out), and the bandwidth those iterations
stand for at the one-pass iteration's 12 words (48 bytes) a row against the
measured HBM copy peak.
Prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

from . import abi, load
from .scene import SceneDesc, pressure_problem


def run(size=256, precision="mixed", iters=300, repeat=3, seed=0):
    import numpy as np
    import torch
    lib = load()
    desc = SceneDesc(N=size)
    minv, diag, b = pressure_problem(desc, seed)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    dm, dd, db = dev(minv), dev(diag), dev(b)
    dx = torch.zeros_like(db)
    g = abi.Grid(desc.res, desc.res, desc.res, desc.dh, (C.c_double * 3)(0, 0, 0))
    prec = {"mixed": abi.ESF_MIXED, "mixed-x64": abi.ESF_MIXED_X64}.get(precision, abi.ESF_FP64)
    stream = torch.cuda.current_stream()
    it, rr = C.c_int(), C.c_double()
    p = lambda t: C.c_void_p(t.data_ptr())

    def solve(n):
        dx.zero_()
        s = lib.esf_pressure_solve(C.byref(g), p(dm), p(dd), p(db), p(dx), 1e-30, n, prec,
                                   C.byref(it), C.byref(rr), C.c_void_p(stream.cuda_stream))
        if s != 0:
            raise abi.EsfError(s, "esf_pressure_solve", (lib.esf_last_error() or b"").decode())
        return it.value

    solve(min(iters, 20))  # warm-up: module load, graph capture
    rates = []
    for _ in range(repeat):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        n = solve(iters)
        e1.record(stream)
        torch.cuda.synchronize()
        rates.append(n / (e0.elapsed_time(e1) * 1e-3))
    R = desc.N ** 3
    return {"metric": "pressure PCR iterations/s", "size": size, "rows": R, "precision": precision,
            "iters_per_solve": n, "iters_per_s": max(rates), "all_iters_per_s": rates,
            "us_per_iter": 1e6 / max(rates)}


def run_batch(size=32, batch=256, iters=300, repeat=2, autotune=False):
    import os
    import time

    import numpy as np
    import torch
    lib = load()
    desc = SceneDesc(N=size)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")
    systems = [pressure_problem(desc, seed) for seed in range(batch)]
    dm = [dev(m) for m, _, _ in systems]
    dd = [dev(d) for _, d, _ in systems]
    db = [dev(b) for _, _, b in systems]
    dx = [torch.zeros_like(b) for b in db]
    grids = (abi.Grid * batch)(*[abi.Grid(desc.res, desc.res, desc.res, desc.dh, (C.c_double * 3)(0, 0, 0))
                                 for _ in range(batch)])
    arr = lambda ts: (C.c_void_p * batch)(*[t.data_ptr() for t in ts])
    its = (C.c_int * batch)()
    rr = (C.c_double * batch)()
    from .serve import BatchStats
    stats = BatchStats()

    def solve(n):
        for x in dx:
            x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = lib.esf_pressure_solve_batch(batch, grids, arr(dm), arr(dd), arr(db), arr(dx), 1e-30, n,
                                         abi.ESF_MIXED, int(autotune), its, rr, C.byref(stats), None)
        t = time.perf_counter() - t0
        if s != 0:
            raise abi.EsfError(s, "esf_pressure_solve_batch", (lib.esf_last_error() or b"").decode())
        return sum(its), t

    solve(min(iters, 20))
    best = None
    for _ in range(repeat):
        n, t = solve(iters)
        if best is None or n / t > best[0] / best[1]:
            best = (n, t)
    n, t = best
    n4, t4 = solve(4 * iters)
    marginal = (n4 - n) / (t4 - t) if t4 > t else None
    kernel = stats.as_dict()
    R = desc.N ** 3
    peak = None
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            peak = float(json.load(f)["hbm_gbs"])
    gbs = n * 48.0 * R / t / 1e9
    mgbs = marginal * 48.0 * R / 1e9 if marginal else None
    return {"metric": "batched pressure PCR iterations/s", "size": size, "batch": batch, "rows_each": R,
            "autotune": autotune,
            "precision": "mixed", "iters_per_solve": iters, "iters_total": n, "wall_s": t,
            "iters_per_s": n / t, "effective_gbs": gbs, "hbm_peak_gbs": peak,
            "frac_of_hbm": (gbs / peak) if peak else None,
            "marginal_iters_per_s": marginal, "marginal_gbs": mgbs,
            "marginal_frac_of_hbm": (mgbs / peak) if (peak and mgbs) else None,
            "launch_ms": kernel["launch_ms"], "launch_gbs": kernel["launch_gbs"],
            "launch_frac_of_hbm": (kernel["launch_gbs"] / peak) if (peak and kernel["launch_gbs"]) else None,
            "tasks_per_launch": kernel["mean_tasks"],
            "what": "wall clock around one esf_pressure_solve_batch call (host threads, work arrays, "
                    "refinements and set-up passes included); bandwidth = iterations x 48 bytes x rows / "
                    "wall; marginal_* from a 4x longer call (per-call set-up left out); launch_* from "
                    "CUDA events around every 8th chunk of batched launches (48 bytes x rows / device time)"}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed-x64", "fp64"])
    ap.add_argument("--iters", type=int, default=300)
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--autotune", action="store_true", help="batched: tune the tile depth by timing")
    a = ap.parse_args(argv)
    if a.batch > 1:
        print(json.dumps(run_batch(a.size, a.batch, a.iters, a.repeat, a.autotune)), flush=True)
    else:
        print(json.dumps(run(a.size, a.precision, a.iters, a.repeat)), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
