"""Serving benchmark: a stream of independent coupled-step scenes arriving as
a Poisson process, served by the multi-scene server (esf_server_*), against
the same scenes run one after another.

Scenes (seeded): grid N uniform from --sizes, sphere radius U[0.08, 0.2] at
(0.5, 0.65, 0.5), fluid height U[0.2, 0.4], E log-uniform in [5e4, 1e6],
nu = 0.45, seeded fluid noise; each request is --steps coupled steps in
mixed precision to the 1e-8 FP64 residual.

    python -m eulersf_gb300.serve_bench [--requests 60] [--rate 40] [--steps 10]
                                        [--seed 11] [--max-active 8] [--no-sequential]
                                        [--no-batching]

Prints one JSON line: scene-steps/s served and sequential, the ratio, and
the p50/p99 request latency (submit to last step). The served run batches
the inner solves of active scenes of one grid shape (continuous batching,
unless --no-batching); the sequential run steps one scene at a time.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import abi
from .scene import SceneDesc, SolidDesc


def make_requests(n, seed, sizes):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(rng.choice(sizes))
        r = float(rng.uniform(0.08, 0.2))
        h = float(rng.uniform(0.2, 0.4))
        E = float(math.exp(rng.uniform(math.log(5e4), math.log(1e6))))
        out.append(SceneDesc(N=N, mass_sample_dh=(1.0 / N) / 4, fluid_height=h, noise_seed=seed * 1000 + i,
                             solids=[SolidDesc(center=(0.5, 0.65, 0.5), radius=r, E=E, nu=0.45)]))
    return out


def serve(descs, steps, rate, seed, max_active, batching=True, autotune=False):
    from .serve import Server
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(descs))) if rate > 0 else np.zeros(len(descs))
    stats = []
    with Server(max_active=max_active, batching=batching, autotune=autotune) as srv:
        t0 = time.perf_counter()
        tickets = []
        for d, at in zip(descs, arrivals):
            now = time.perf_counter() - t0
            if at > now:
                time.sleep(at - now)
            tickets.append(srv.submit(d, steps, abi.ESF_MIXED))
        for t in tickets:
            st = srv.wait(t)
            if st["state"] != 2:
                raise RuntimeError(f"request {t} failed: {st}")
            stats.append(st)
            srv.release(t)
        wall = time.perf_counter() - t0
        batch = srv.batch_stats()
    return wall, stats, batch


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=60)
    ap.add_argument("--rate", type=float, default=40.0)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--sizes", default="48,64,96,128,160")
    ap.add_argument("--max-active", type=int, default=8)
    ap.add_argument("--no-sequential", action="store_true")
    ap.add_argument("--autotune", action="store_true", help="tune each batch lane's tile depth by timing")
    ap.add_argument("--no-batching", action="store_true",
                    help="each scene's inner solves on its own stream (no shared launches)")
    a = ap.parse_args(argv)
    descs = make_requests(a.requests, a.seed, [int(x) for x in a.sizes.split(",")])
    wall, stats, batch = serve(descs, a.steps, a.rate, a.seed, a.max_active, not a.no_batching, a.autotune)
    lat = np.array([s["latency_ms"] for s in stats])
    steps_all = a.steps * len(descs)
    line = {"metric": "served scene-steps/s (Poisson arrivals)", "requests": len(descs),
            "rate_per_s": a.rate, "steps_per_request": a.steps, "max_active": a.max_active,
            "sizes": a.sizes, "served_steps_per_s": steps_all / wall, "served_wall_s": wall,
            "latency_p50_ms": float(np.percentile(lat, 50)), "latency_p99_ms": float(np.percentile(lat, 99)),
            "queued_p50_ms": float(np.percentile([s["queued_ms"] for s in stats], 50)),
            "max_rel_residual": max(max(s["last"]["rel_residual"]) for s in stats),
            "batching": not a.no_batching, "autotune": a.autotune, "batch_stats": batch}
    if not a.no_sequential:
        swall, sstats, _ = serve(descs, a.steps, 0.0, a.seed, 1, False)
        line["sequential_steps_per_s"] = steps_all / swall
        line["sequential_wall_s"] = swall
        line["served_over_sequential"] = line["served_steps_per_s"] / line["sequential_steps_per_s"]
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
