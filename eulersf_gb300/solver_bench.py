"""Pressure-solver throughput through the solver seam (esf_pressure_solve,
the replacement of CONJUGATE_RESIDUAL::solvePCR with getMatVecMult,
CONJUGATE_RESIDUAL.inl:109-192, COUPLED_INTEGRATOR_3D.cpp:638-660): PCR
iterations per second ("CG iters/s") on a pressure system of the rubber-ball
scene's size, device-resident inputs, timed with CUDA events on the stream
the solve runs on.

    python -m eulersf_gb300.solver_bench [--size 256] [--precision mixed|fp64]
                                         [--iters 300] [--repeat 3]

The tolerance is set to 1e-30 so every solve runs exactly --iters
iterations (mixed: FP32 inner iterations summed over the refinements).
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
    prec = abi.ESF_MIXED if precision == "mixed" else abi.ESF_FP64
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


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--iters", type=int, default=300)
    ap.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args(argv)
    print(json.dumps(run(a.size, a.precision, a.iters, a.repeat)), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
